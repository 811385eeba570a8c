// Hockney doubled-grid Poisson plan and batched pair solves (internal API).
#pragma once
#include "common.cuh"
#include "fft.cuh"

namespace gato {

constexpr int kMaxIn = 12;      // input fields a pass can read (orbitals, psi, rho)
constexpr int kMaxOut = 8;      // output fields a pass can accumulate into
constexpr int kMaxFields = 40;  // complex fields (= two real densities) per call

// One real density packed into the real or imaginary part of a complex field,
// and what the epilogue does with its potential J.
struct PartDesc {
  int8_t a = -1, b = -1;          // density = in[a] * in[b] (b < 0: in[a]); a < 0: unused
  int8_t nt = 0;                  // accumulation terms
  int8_t to[2] = {0, 0};          // out[to] += coef * in[tc] * J   (tc < 0: * 1)
  int8_t tc[2] = {-1, -1};
  int8_t eslot = 0;               // energy mode: slot += ew * density * J
  float coef[2] = {0.f, 0.f};
  double ew = 0.0;
};
struct FieldDesc {
  PartDesc p[2];
};
struct PassArgs {
  const void* in[kMaxIn] = {};
  void* out[kMaxOut] = {};
  int nout = 0;
  int nf = 0;
  FieldDesc f[kMaxFields];
  // EPI_J: part k (= 2 * field + {0: real, 1: imaginary}) of J is written to
  // jbase + k * jstride
  void* jbase = nullptr;
  int64_t jstride = 0;
};

struct PoissonPlan {
  int dtype = GATO_F64;
  int N = 0, M = 0, H = 0;
  int max_fields = 0;
  double h = 0, eps = 0, dV = 0;
  FftPlanDev fp{};
  void* ghat = nullptr;    // H^3 octant of the kernel spectrum, x dV / M^3
  void* tw = nullptr;      // M twiddles exp(-2 pi i k / M)
  void* tw2 = nullptr;     // register engine: tw2[k1 S + n2] = exp(-2 pi i n2 k1 / M), M = R1 R2,
                           // S = fft2::tw_row_stride
  void* tw4 = nullptr;     // packed FP32 engine: tw4[k1 R2 + n2] = (c, c, s, s), (c, s) = exp(-2 pi i n2 k1 / M)
  void* ghat2 = nullptr;   // packed FP32 engine: kernel spectrum folded in x and y only, [kxo][kyo][kz < M]
  void* S1 = nullptr;      // max_fields x N x N x M complex
  void* S2 = nullptr;      // max_fields x N x M x M complex
  double* partials = nullptr;
  int npart_cap = 0;
  int group = 0;           // fields per launch group (0: max_fields)
  int engine = 0;          // 0: register two-pass kernels where M allows, 1: generic Stockham
                           // (2, 3: z-forward variants; 4: as 0 with the scalar column passes)
};

enum PoissonEpi { EPI_ACC = 0, EPI_ENERGY = 1, EPI_J = 2 };

enum ColMode { COL_FWD = 0, COL_INV = 1, COL_FMI = 2 };

// Geometry of a batched strided-line pass over [field][outer][pos][col].
struct ColGeom {
  int64_t in_fs, out_fs;   // field strides (elements)
  int64_t in_os, out_os;   // outer strides
  int64_t in_ps, out_ps;   // position strides
  int ncols;               // contiguous columns (lines)
  int nin, nout;           // input positions, output positions kept
};

template <typename T>
__device__ __forceinline__ T dens(const PartDesc& d, const void* const* in, int64_t gi) {
  T v = reinterpret_cast<const T*>(in[d.a])[gi];
  if (d.b >= 0) v *= reinterpret_cast<const T*>(in[d.b])[gi];
  return v;
}

// Weights of the spectral (Parseval) energy pass: field f of a call adds
// w[f] * sum_k ghat(k) |F_f(k)|^2 to energy slot slot[f]. Partials are laid
// out [slot][field][y block][x block] of the x-pass grid, slot_stride entries
// per slot.
struct FeArgs {
  double* partials = nullptr;
  int64_t slot_stride = 0;
  int f0 = 0;                  // first field of this launch within the call
  double w[kMaxFields] = {};
  int8_t slot[kMaxFields] = {};
};

// Register-resident two-pass kernels for the common sizes M = 2N (see
// fft2.cuh); each returns kNotHandled when M has no instantiation.
namespace fast {
constexpr int kNotHandled = 1;
template <typename T> int rows_L(int M);   // lines per CTA of the z kernels, 0 if unsupported
int shape_r2(int M);                        // R2 of the register engine's M = R1 R2, 0 if none
template <typename T>
int cols(int M, int mode, const typename Cplx<T>::type* in, typename Cplx<T>::type* out,
         const ColGeom& g, int outer, int nf, const typename Cplx<T>::type* tw, const T* ghat,
         int H, cudaStream_t s);
// FP32 column passes on the packed two-line engine (poisson_packed.cuh): R2 of
// M = R1 R2 when M has an instantiation, else 0.
int packed_r2(int M);
int packed_cols(int M, int mode, const float2* in, float2* out, const ColGeom& g, int outer, int nf,
                const float4* tw4, const float* ghat2, int H, cudaStream_t s);
// x forward of the y-transformed fields and the kernel-weighted spectral power
// per CTA (the energy epilogue without the inverse passes).
template <typename T>
int cols_fe(int M, const typename Cplx<T>::type* in, const ColGeom& g, int outer, int nf,
            const typename Cplx<T>::type* tw, const T* ghat, int H, const FeArgs& fa,
            cudaStream_t s);
template <typename T>
int rows_fwd(int M, const PassArgs& a, int f0, int nfg, typename Cplx<T>::type* S1,
             const typename Cplx<T>::type* tw, int multi, cudaStream_t s);
template <typename T>
int rows_inv(int M, const PassArgs& a, int f0, int nfg, const typename Cplx<T>::type* S1,
             const typename Cplx<T>::type* tw, int accumulate, bool energy, double* partials,
             int64_t slot_stride, cudaStream_t s);
// z inverse writing the real and imaginary parts of J as separate fields (EPI_J).
template <typename T>
int rows_inv_j(int M, const PassArgs& a, int f0, int nfg, const typename Cplx<T>::type* S1,
               const typename Cplx<T>::type* tw, cudaStream_t s);
}  // namespace fast

// out_a -= phi_b J_ab and out_b -= phi_a J_ab for every pair a <= b of n
// fields, J_ab the k-th field of J in row-major pair order (0,0),(0,1),...
int pair_exchange(int dtype, const void* orbitals, int n, const void* J, void* out, int64_t n3,
                  cudaStream_t s);
// True when the plan's size has register-engine kernels (EPI_J available).
bool poisson_j_supported(const PoissonPlan& pl);
// True when energies take the spectral (Parseval) pass: FP64 plans on the
// register engine. FP32 energies keep the full solves (their share of a mixed
// SCF is small, and their rounding is the one the FP32 energy terms were
// validated with).
bool poisson_fe_supported(const PoissonPlan& pl);

// Runs every field of `args` through the pair-solve pipeline in groups of
// at most plan.max_fields. EPI_ACC: out[o] = (accumulate ? out[o] : 0) +
// sum of terms. EPI_ENERGY: energy_dev[slot] = dV * sum of weighted terms
// (two slots).
// join (EPI_ACC only, may be null): the stream waits on it before the first z-inverse epilogue,
// the first kernel that reads or writes the outputs (work on another stream that also writes them,
// ordered before the accumulation without holding up the transforms).
int poisson_run(PoissonPlan& pl, const PassArgs& args, int epi, bool accumulate,
                double* energy_dev, cudaStream_t s, cudaEvent_t join = nullptr);

}  // namespace gato

struct gato_poisson_plan {
  gato::PoissonPlan p;
};
