// Register-resident two-pass FFT engine for line lengths M = R1 * R2.
//
// A CTA transforms L lines at once; each thread owns one line of one stage
// and keeps its R1 or R2 points in registers. With n = R2 n1 + n2 and
// k = k1 + R1 k2 the DFT factors as (the "four-step" decomposition)
//   X[k1 + R1 k2] = sum_n2 W_R2^{n2 k2} W_M^{n2 k1} sum_n1 W_R1^{n1 k1} x[R2 n1 + n2]
// stage 1: thread (line, n2) does the R1-point DFT over n1 (stride R2);
// stage 2: thread (line, k1) applies W_M^{n2 k1} and the R2-point DFT over
// n2, leaving X[k1 + R1 k2] in its registers. The inverse runs the same
// factorisation backwards from that register layout, so a forward transform,
// a pointwise multiply and an inverse transform cost two shared-memory round
// trips in total. The in-register DFTs are unrolled with compile-time
// twiddles (twiddles.cuh). The first N = M/2 inputs are the only nonzero
// ones in the zero-padded forward transforms (R1 is even, so they are
// n1 < R1/2), and the inverse keeps only the first M/2 outputs.
#pragma once
#include "fft.cuh"
#include "twiddles.cuh"

namespace gato {
namespace fft2 {

template <int R> struct Split;
template <> struct Split<6> { static constexpr int A = 2, B = 3; };
template <> struct Split<10> { static constexpr int A = 2, B = 5; };
template <> struct Split<12> { static constexpr int A = 4, B = 3; };
template <> struct Split<14> { static constexpr int A = 2, B = 7; };
template <> struct Split<16> { static constexpr int A = 4, B = 4; };
template <> struct Split<20> { static constexpr int A = 4, B = 5; };
template <> struct Split<24> { static constexpr int A = 8, B = 3; };

// a * exp(DIR * 2 pi i e / R), e a compile-time constant after unrolling
template <typename T2, int R, int DIR>
__device__ __forceinline__ T2 ctw(T2 a, int e) {
  using Rt = typename CT<T2>::R;
  if (e == 0) return a;
  if ((4 * e) % R == 0) {   // a quarter-turn multiple: -1 or +-i, exact sign and swap
    const int k = 4 * e / R;
    T2 r;
    if (k == 2) {
      r.x = -a.x;
      r.y = -a.y;
    } else if ((k == 1) == (DIR > 0)) {   // * i
      r.x = -a.y;
      r.y = a.x;
    } else {                              // * -i
      r.x = a.y;
      r.y = -a.x;
    }
    return r;
  }
  const Rt c = (Rt)TwC<R>::c(e);
  const Rt s = (Rt)DIR * (Rt)TwC<R>::s(e);
  T2 r;
  r.x = a.x * c - a.y * s;
  r.y = a.x * s + a.y * c;
  return r;
}

// In-place R-point DFT in natural order; DIR = -1 forward, +1 inverse (unscaled).
template <typename T2, int R, int DIR>
__device__ __forceinline__ void rdft(T2* v) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    dft2(v);
  } else if constexpr (R == 4) {
    dft4(v[0], v[1], v[2], v[3], DIR);
  } else if constexpr (R == 8) {
    dft8(v, DIR);
  } else if constexpr (R == 3 || R == 5 || R == 7) {
    dft_odd<T2, R>(v, DIR);
  } else {
    constexpr int A = Split<R>::A, B = Split<R>::B;
    T2 y[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      T2 u[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) u[n1] = v[B * n1 + n2];
      rdft<T2, A, DIR>(u);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = ctw<T2, R, DIR>(u[k1], (n2 * k1) % R);
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      T2 u[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) u[n2] = y[n2 * A + k1];
      rdft<T2, B, DIR>(u);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
    }
  }
}

// The same DFT when only v[0 .. R/2) is nonzero (the zero-padded half of a
// Hockney transform). For R = A B with A even the zeros are the upper half of
// every inner A-point DFT, so the saving recurses down to the base radices.
template <typename T2, int R, int DIR>
__device__ __forceinline__ void rdft_half(T2* v) {
  if constexpr (R == 2) {
    v[1] = v[0];
  } else if constexpr (R == 4) {
    const T2 a = v[0], b = v[1];
    const T2 ib = cmul_i(b, DIR);
    v[0] = cadd(a, b);
    v[1] = cadd(a, ib);
    v[2] = csub(a, b);
    v[3] = csub(a, ib);
  } else if constexpr (R == 8) {
    // even/odd split: E = DFT4(v0, v2, 0, 0), O = DFT4(v1, v3, 0, 0)
    T2 e[4] = {v[0], v[2], v[0], v[0]}, o[4] = {v[1], v[3], v[1], v[1]};
    rdft_half<T2, 4, DIR>(e);
    rdft_half<T2, 4, DIR>(o);
    using Rt = typename CT<T2>::R;
    const Rt s = (Rt)0.70710678118654752440;
    T2 w1, w3;
    w1.x = s;
    w1.y = (Rt)DIR * s;
    w3.x = -s;
    w3.y = (Rt)DIR * s;
    o[1] = cmul(o[1], w1);
    o[2] = cmul_i(o[2], DIR);
    o[3] = cmul(o[3], w3);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[q] = cadd(e[q], o[q]);
      v[q + 4] = csub(e[q], o[q]);
    }
  } else {
    constexpr int A = Split<R>::A, B = Split<R>::B;
    static_assert(A % 2 == 0, "half-input DFT needs an even inner radix");
    T2 y[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      T2 u[A];
#pragma unroll
      for (int n1 = 0; n1 < A / 2; ++n1) u[n1] = v[B * n1 + n2];
      rdft_half<T2, A, DIR>(u);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = ctw<T2, R, DIR>(u[k1], (n2 * k1) % R);
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      T2 u[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) u[n2] = y[n2 * A + k1];
      rdft<T2, B, DIR>(u);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
    }
  }
}

template <int R1, int R2> struct Shape {
  static constexpr int M = R1 * R2;
  static constexpr int RMAX = R1 > R2 ? R1 : R2;
};

// Row stride, in entries, of the stage-twiddle table
// tw[k1 * stride + n2] = exp(-2 pi i n2 k1 / M) (R1 rows). Consecutive lanes
// of the row passes read consecutive rows: the padding puts those rows in
// distinct shared-memory banks (FP32 twiddles move in 16-byte pairs, so a row
// starts on a 16-byte boundary; FP64 twiddles are one 16-byte load each).
__host__ __device__ constexpr int tw_row_stride(bool f32, int R2) {
  return f32 ? ((R2 / 2) % 2 == 0 ? R2 + 2 : R2) : R2 + 1;
}
template <typename T2, int R2> struct TwRow {
  static constexpr int S = tw_row_stride(sizeof(T2) == 8, R2);
};

// a * w for w = (c, s) = exp(-2 pi i e / M) (DIR = -1) or its conjugate (DIR = +1).
template <typename T2, int DIR>
__device__ __forceinline__ T2 rtw(T2 a, typename CT<T2>::R c, typename CT<T2>::R s) {
  T2 w;
  w.x = c;
  w.y = DIR > 0 ? -s : s;
  return cmul(a, w);
}

// X[n2] *= W_M^{DIR n2 k1} for n2 = 1 .. R2-1 from row k1 of the stage table,
// row[n2] = exp(-2 pi i n2 k1 / M). The row is contiguous, so float twiddles
// come in pairs from one 16-byte shared load (R2 is even and every row starts
// on a 16-byte boundary); n2 = 0 is the identity and skipped.
template <typename T2, int R2, int DIR>
__device__ __forceinline__ void twiddle_row(T2* X, const T2* row) {
  if constexpr (sizeof(T2) == 8) {
    static_assert(R2 % 2 == 0, "paired twiddle loads need an even R2");
    const float4* r4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int p = 0; p < R2 / 2; ++p) {
      const float4 w = r4[p];
      if (p > 0) X[2 * p] = rtw<T2, DIR>(X[2 * p], w.x, w.y);
      X[2 * p + 1] = rtw<T2, DIR>(X[2 * p + 1], w.z, w.w);
    }
  } else {
#pragma unroll
    for (int n2 = 1; n2 < R2; ++n2) X[n2] = rtw<T2, DIR>(X[n2], row[n2].x, row[n2].y);
  }
}

// Stage 1 of the forward transform for the item (line, n2): reads x[R2 n1 + n2]
// through `get` (only n1 < R1/2 when HALF), writes Y[n2][k1] to buf.
template <typename T2, int R1, int R2, bool HALF, typename Get>
__device__ __forceinline__ void fwd_stage1(T2* buf, int LP, int line, int n2, Get get) {
  T2 v[R1];
#pragma unroll
  for (int n1 = 0; n1 < R1; ++n1) {
    if (!HALF || n1 < R1 / 2) v[n1] = get(R2 * n1 + n2);
    else v[n1].x = v[n1].y = 0;
  }
  if constexpr (HALF) rdft_half<T2, R1, -1>(v);
  else rdft<T2, R1, -1>(v);
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) buf[(n2 * R1 + k1) * LP + line] = v[k1];
}

// Stage 2 of the forward transform for (line, k1): X[k2] = spectrum at k1 + R1 k2.
// tw is the stage-twiddle table (R1 rows, see tw_row_stride).
template <typename T2, int R1, int R2>
__device__ __forceinline__ void fwd_stage2(const T2* buf, int LP, int line, int k1, const T2* tw,
                                           T2* X) {
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) X[n2] = buf[(n2 * R1 + k1) * LP + line];
  twiddle_row<T2, R2, -1>(X, tw + k1 * TwRow<T2, R2>::S);
  rdft<T2, R2, -1>(X);
}

// Inverse stage A for (line, k1) holding X[k2] = spectrum at k1 + R1 k2: writes Z to buf.
template <typename T2, int R1, int R2>
__device__ __forceinline__ void inv_stageA(T2* buf, int LP, int line, int k1, const T2* tw, T2* X) {
  rdft<T2, R2, +1>(X);
  twiddle_row<T2, R2, +1>(X, tw + k1 * TwRow<T2, R2>::S);
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) buf[(n2 * R1 + k1) * LP + line] = X[n2];
}

// Inverse stage B for (line, n2): outputs x[n2 + R2 n1] through `put` (n1 < R1/2 when HALF).
template <typename T2, int R1, int R2, bool HALF, typename Put>
__device__ __forceinline__ void inv_stageB(const T2* buf, int LP, int line, int n2, Put put) {
  T2 w[R1];
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) w[k1] = buf[(n2 * R1 + k1) * LP + line];
  rdft<T2, R1, +1>(w);
#pragma unroll
  for (int n1 = 0; n1 < R1; ++n1)
    if (!HALF || n1 < R1 / 2) put(n2 + R2 * n1, w[n1]);
}

// ---- row passes (the contiguous z axis) ----------------------------------------
// Line `line`'s stage element (n2, k1) sits at line * LS + n2 * (R1 + 1) + k1.
// Stages 1 and B run with n2 across the lanes, stages 2 and A with k1 across
// the lanes: both orders walk the buffer with odd element strides (no bank
// conflicts), stage 2 leaves spectrum entries k1 + R1 k2 that consecutive
// lanes store to consecutive addresses, and stage B leaves outputs
// n2 + R2 n1 in the same coalesced order, so no transpose through shared
// memory is needed on either side.
template <int R1, int R2> struct RowBuf {
  static constexpr int LS = R2 * (R1 + 1);
  static __device__ __forceinline__ int at(int line, int n2, int k1) {
    return line * LS + n2 * (R1 + 1) + k1;
  }
};

// Stage 1 for (line, n2): v[n1] = x[R2 n1 + n2] (n1 < R1/2 only when HALF).
template <typename T2, int R1, int R2, bool HALF>
__device__ __forceinline__ void row_fwd_stage1(T2* buf, int line, int n2, T2* v) {
  if constexpr (HALF) {
#pragma unroll
    for (int n1 = R1 / 2; n1 < R1; ++n1) v[n1].x = v[n1].y = 0;
    rdft_half<T2, R1, -1>(v);
  } else {
    rdft<T2, R1, -1>(v);
  }
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) buf[RowBuf<R1, R2>::at(line, n2, k1)] = v[k1];
}

// Stage 2 for (line, k1): X[k2] = spectrum at k1 + R1 k2.
template <typename T2, int R1, int R2>
__device__ __forceinline__ void row_fwd_stage2(const T2* buf, int line, int k1, const T2* tw, T2* X) {
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) X[n2] = buf[RowBuf<R1, R2>::at(line, n2, k1)];
  twiddle_row<T2, R2, -1>(X, tw + k1 * TwRow<T2, R2>::S);
  rdft<T2, R2, -1>(X);
}

// Inverse stage A for (line, k1) holding X[k2] = spectrum at k1 + R1 k2.
template <typename T2, int R1, int R2>
__device__ __forceinline__ void row_inv_stageA(T2* buf, int line, int k1, const T2* tw, T2* X) {
  rdft<T2, R2, +1>(X);
  twiddle_row<T2, R2, +1>(X, tw + k1 * TwRow<T2, R2>::S);
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) buf[RowBuf<R1, R2>::at(line, n2, k1)] = X[n2];
}

// Inverse stage B for (line, n2): w[n1] = output at z = n2 + R2 n1.
template <typename T2, int R1, int R2>
__device__ __forceinline__ void row_inv_stageB(const T2* buf, int line, int n2, T2* w) {
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) w[k1] = buf[RowBuf<R1, R2>::at(line, n2, k1)];
  rdft<T2, R1, +1>(w);
}

}  // namespace fft2
}  // namespace gato
