// Instantiations of the register-resident pair-solve kernels for float fields.
// Table: M = 2N -> (R1, R2, lines per CTA); R1 is even so the zero-padded
// half of every transform maps to whole register slots.
#include "poisson_packed.cuh"

namespace gato {
namespace fast {

#define GATO_FAST_SHAPES(X)                                                              \
  X(32, 4, 8, 32, 16) X(48, 6, 8, 32, 16) X(64, 8, 8, 32, 16) X(80, 10, 8, 32, 16)      \
  X(96, 8, 12, 16, 8) X(128, 8, 16, 16, 8) X(160, 10, 16, 16, 8) X(192, 12, 16, 16, 8) \
  X(256, 16, 16, 16, 8) X(320, 20, 16, 16, 8)

using T = float;
using T2 = typename Cplx<T>::type;
constexpr bool kF32 = sizeof(T) == 4;

int shape_r2(int M) {
#define X(MM, A, B, L32, L64) \
  case MM: return B;
  switch (M) { GATO_FAST_SHAPES(X) }
#undef X
  return 0;
}

template <>
int rows_L<T>(int M) {
#define X(MM, A, B, L32, L64) \
  case MM: return kF32 ? L32 : L64;
  switch (M) { GATO_FAST_SHAPES(X) }
#undef X
  return 0;
}

template <>
int cols<T>(int M, int mode, const T2* in, T2* out, const ColGeom& g, int outer, int nf, const T2* tw,
            const T* ghat, int H, cudaStream_t s) {
#define X(MM, A, B, L32, L64) \
  case MM: return Launch<T, A, B, kF32 ? L32 : L64>::cols(mode, in, out, g, outer, nf, tw, ghat, H, s);
  switch (M) { GATO_FAST_SHAPES(X) }
#undef X
  return kNotHandled;
}

template <>
int rows_fwd<T>(int M, const PassArgs& a, int f0, int nfg, T2* S1, const T2* tw, int multi, cudaStream_t s) {
#define X(MM, A, B, L32, L64) \
  case MM: return Launch<T, A, B, kF32 ? L32 : L64>::rows_fwd(a, f0, nfg, S1, tw, multi, s);
  switch (M) { GATO_FAST_SHAPES(X) }
#undef X
  return kNotHandled;
}

template <>
int rows_inv<T>(int M, const PassArgs& a, int f0, int nfg, const T2* S1, const T2* tw, int accumulate,
                bool energy, double* partials, int64_t slot_stride, cudaStream_t s) {
#define X(MM, A, B, L32, L64)                                                             \
  case MM:                                                                                \
    return Launch<T, A, B, kF32 ? L32 : L64>::rows_inv(a, f0, nfg, S1, tw, accumulate, energy, \
                                                       partials, slot_stride, s);
  switch (M) { GATO_FAST_SHAPES(X) }
#undef X
  return kNotHandled;
}

template <>
int rows_inv_j<T>(int M, const PassArgs& a, int f0, int nfg, const T2* S1, const T2* tw, cudaStream_t s) {
#define X(MM, A, B, L32, L64) \
  case MM: return Launch<T, A, B, kF32 ? L32 : L64>::rows_inv_j(a, f0, nfg, S1, tw, s);
  switch (M) { GATO_FAST_SHAPES(X) }
#undef X
  return kNotHandled;
}

// Packed two-line column passes: M -> (R1, R2), 8 line pairs per CTA.
#define GATO_PACKED_SHAPES(X) X(128, 8, 16) X(160, 10, 16) X(192, 12, 16) X(256, 16, 16) X(320, 20, 16)

int packed_r2(int M) {
#define X(MM, A, B) \
  case MM: return B;
  switch (M) { GATO_PACKED_SHAPES(X) }
#undef X
  return 0;
}

int packed_cols(int M, int mode, const float2* in, float2* out, const ColGeom& g, int outer, int nf,
                const float4* tw4, const float* ghat2, int H, cudaStream_t s) {
#define X(MM, A, B) \
  case MM: return packed::LaunchP<A, B, 8>::cols(mode, in, out, g, outer, nf, tw4, ghat2, s);
  switch (M) { GATO_PACKED_SHAPES(X) }
#undef X
  return kNotHandled;
}

}  // namespace fast
}  // namespace gato
