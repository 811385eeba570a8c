// Packed two-line FP32 variant of the register-resident two-pass FFT engine.
//
// GB300 (sm_103) issues FP32 adds, multiplies and FMAs on register pairs
// (add/sub/mul/fma .f32x2): one instruction performs the same operation on
// two independent lanes of data. The strided-line passes of the Poisson
// pipeline are instruction-issue bound on their radix-16 DFTs, so here each
// thread transforms TWO lines at once and keeps every value of a position as
// a pair: CP{re = (re_a, re_b), im = (im_a, im_b)} for lines a and b. Every
// complex add, subtract and multiply by a shared twiddle then costs half the
// instructions of the scalar engine (fft2.cuh), which this file mirrors
// stage for stage (same factorisation, same twiddles, same pruning).
//
// Multiplications by +-i are never formed on their own (they would need a
// data-dependent negation); the DFT kernels fold them into the following
// add/subtract by swapping real and imaginary parts and exchanging add and
// subtract. Constant twiddles are register pairs (c, c) / (s, s).
#pragma once
#include "fft2.cuh"

namespace gato {
namespace fft2p {

struct CP {
  float2 re, im;
};

union U64F2 {
  float2 f;
  unsigned long long u;
};

__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) {
  U64F2 x, y, d;
  x.f = a;
  y.f = b;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.u) : "l"(x.u), "l"(y.u));
  return d.f;
}
__device__ __forceinline__ float2 pneg(float2 a) { return psub(make_float2(0.f, 0.f), a); }
__device__ __forceinline__ float2 pk(float c) { return make_float2(c, c); }

__device__ __forceinline__ CP cadd(const CP& a, const CP& b) { return {padd(a.re, b.re), padd(a.im, b.im)}; }
__device__ __forceinline__ CP csub(const CP& a, const CP& b) { return {psub(a.re, b.re), psub(a.im, b.im)}; }

// a + DIR*i*b and a - DIR*i*b without forming i*b
template <int DIR>
__device__ __forceinline__ void bfly_i(const CP& a, const CP& b, CP& plus, CP& minus) {
  if (DIR < 0) {   // -i b = (b.im, -b.re)
    plus = {padd(a.re, b.im), psub(a.im, b.re)};
    minus = {psub(a.re, b.im), padd(a.im, b.re)};
  } else {         // +i b = (-b.im, b.re)
    plus = {psub(a.re, b.im), padd(a.im, b.re)};
    minus = {padd(a.re, b.im), psub(a.im, b.re)};
  }
}

// a * (c + i s) for a compile-time (c, s)
__device__ __forceinline__ CP cmul_k(const CP& a, float c, float s) {
  return {pfma(a.re, pk(c), pmul(a.im, pk(-s))), pfma(a.re, pk(s), pmul(a.im, pk(c)))};
}

// a * exp(DIR * 2 pi i e / R), e a compile-time constant after unrolling
template <int R, int DIR>
__device__ __forceinline__ CP ctw(const CP& a, int e) {
  if (e == 0) return a;
  if ((4 * e) % R == 0) {
    const int k = 4 * e / R;
    if (k == 2) return {pneg(a.re), pneg(a.im)};
    if ((k == 1) == (DIR > 0)) return {pneg(a.im), a.re};   // * i
    return {a.im, pneg(a.re)};                             // * -i
  }
  const float c = (float)TwC<R>::c(e);
  const float s = (float)DIR * (float)TwC<R>::s(e);
  return cmul_k(a, c, s);
}

template <int DIR>
__device__ __forceinline__ void dft2(CP* v) {
  const CP a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int DIR>
__device__ __forceinline__ void dft4(CP& v0, CP& v1, CP& v2, CP& v3) {
  const CP t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), d = csub(v1, v3);
  v0 = cadd(t0, t2);
  v2 = csub(t0, t2);
  bfly_i<DIR>(t1, d, v1, v3);
}

template <int DIR>
__device__ __forceinline__ void dft8(CP* v) {
  CP e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  CP o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<DIR>(e0, e1, e2, e3);
  dft4<DIR>(o0, o1, o2, o3);
  const float2 S = pk(0.70710678118654752440f), NS = pk(-0.70710678118654752440f);
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  bfly_i<DIR>(e2, o2, v[2], v[6]);
  if (DIR < 0) {
    // o1 * exp(-i pi/4) = s (o1.re + o1.im, o1.im - o1.re)
    const float2 A = padd(o1.re, o1.im), B = psub(o1.im, o1.re);
    v[1] = {pfma(A, S, e1.re), pfma(B, S, e1.im)};
    v[5] = {pfma(A, NS, e1.re), pfma(B, NS, e1.im)};
    // o3 * exp(-3 i pi/4) = s (o3.im - o3.re, -(o3.re + o3.im))
    const float2 C = psub(o3.im, o3.re), D = padd(o3.re, o3.im);
    v[3] = {pfma(C, S, e3.re), pfma(D, NS, e3.im)};
    v[7] = {pfma(C, NS, e3.re), pfma(D, S, e3.im)};
  } else {
    // o1 * exp(i pi/4) = s (o1.re - o1.im, o1.re + o1.im)
    const float2 A = psub(o1.re, o1.im), B = padd(o1.re, o1.im);
    v[1] = {pfma(A, S, e1.re), pfma(B, S, e1.im)};
    v[5] = {pfma(A, NS, e1.re), pfma(B, NS, e1.im)};
    // o3 * exp(3 i pi/4) = s (-(o3.re + o3.im), o3.re - o3.im)
    const float2 C = padd(o3.re, o3.im), D = psub(o3.re, o3.im);
    v[3] = {pfma(C, NS, e3.re), pfma(D, S, e3.im)};
    v[7] = {pfma(C, S, e3.re), pfma(D, NS, e3.im)};
  }
}

// y_k = sum_n x_n exp(DIR 2 pi i n k / 3)
template <int DIR>
__device__ __forceinline__ void dft3(CP* v) {
  const CP s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const CP t = {pfma(s.re, pk(-0.5f), v[0].re), pfma(s.im, pk(-0.5f), v[0].im)};
  const CP u = {pmul(d.re, pk(0.86602540378443864676f)), pmul(d.im, pk(0.86602540378443864676f))};
  v[0] = cadd(v[0], s);
  bfly_i<DIR>(t, u, v[1], v[2]);
}

// y_k = sum_n x_n exp(DIR 2 pi i n k / 5): pairs P_n = x_n + x_{5-n}, D_n = x_n - x_{5-n}
template <int DIR>
__device__ __forceinline__ void dft5(CP* v) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
  const CP P1 = cadd(v[1], v[4]), P2 = cadd(v[2], v[3]), D1 = csub(v[1], v[4]), D2 = csub(v[2], v[3]);
  const CP x0 = v[0];
  v[0] = cadd(x0, cadd(P1, P2));
  // k = 1: A = x0 + c1 P1 + c2 P2, B = s1 D1 + s2 D2; k = 2: A = x0 + c2 P1 + c1 P2, B = s2 D1 - s1 D2
  const CP A1 = {pfma(P2.re, pk(c2), pfma(P1.re, pk(c1), x0.re)), pfma(P2.im, pk(c2), pfma(P1.im, pk(c1), x0.im))};
  const CP B1 = {pfma(D2.re, pk(s2), pmul(D1.re, pk(s1))), pfma(D2.im, pk(s2), pmul(D1.im, pk(s1)))};
  const CP A2 = {pfma(P2.re, pk(c1), pfma(P1.re, pk(c2), x0.re)), pfma(P2.im, pk(c1), pfma(P1.im, pk(c2), x0.im))};
  const CP B2 = {pfma(D2.re, pk(-s1), pmul(D1.re, pk(s2))), pfma(D2.im, pk(-s1), pmul(D1.im, pk(s2)))};
  bfly_i<DIR>(A1, B1, v[1], v[4]);
  bfly_i<DIR>(A2, B2, v[2], v[3]);
}

// In-place R-point DFT of both lines, natural order; DIR = -1 forward, +1 inverse (unscaled).
template <int R, int DIR>
__device__ __forceinline__ void rdft(CP* v) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    dft2<DIR>(v);
  } else if constexpr (R == 3) {
    dft3<DIR>(v);
  } else if constexpr (R == 4) {
    dft4<DIR>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 5) {
    dft5<DIR>(v);
  } else if constexpr (R == 8) {
    dft8<DIR>(v);
  } else {
    constexpr int A = fft2::Split<R>::A, B = fft2::Split<R>::B;
    CP y[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      CP u[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) u[n1] = v[B * n1 + n2];
      rdft<A, DIR>(u);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = ctw<R, DIR>(u[k1], (n2 * k1) % R);
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      CP u[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) u[n2] = y[n2 * A + k1];
      rdft<B, DIR>(u);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
    }
  }
}

// The same DFT when only v[0 .. R/2) is nonzero (the zero-padded half of a
// Hockney transform); R = A B with A even, the saving recursing into the
// inner A-point DFTs (fft2::rdft_half restated on pairs).
template <int R, int DIR>
__device__ __forceinline__ void rdft_half(CP* v) {
  if constexpr (R == 2) {
    v[1] = v[0];
  } else if constexpr (R == 4) {
    const CP a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[2] = csub(a, b);
    bfly_i<DIR>(a, b, v[1], v[3]);
  } else if constexpr (R == 8) {
    // even/odd split: E = DFT4(v0, v2, 0, 0), O = DFT4(v1, v3, 0, 0)
    CP e[4] = {v[0], v[2], v[0], v[0]}, o[4] = {v[1], v[3], v[1], v[1]};
    rdft_half<4, DIR>(e);
    rdft_half<4, DIR>(o);
    const float s = 0.70710678118654752440f;
    o[1] = cmul_k(o[1], s, (float)DIR * s);
    o[3] = cmul_k(o[3], -s, (float)DIR * s);
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o[1]);
    v[5] = csub(e[1], o[1]);
    bfly_i<DIR>(e[2], o[2], v[2], v[6]);
    v[3] = cadd(e[3], o[3]);
    v[7] = csub(e[3], o[3]);
  } else {
    constexpr int A = fft2::Split<R>::A, B = fft2::Split<R>::B;
    static_assert(A % 2 == 0, "half-input DFT needs an even inner radix");
    CP y[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      CP u[A];
#pragma unroll
      for (int n1 = 0; n1 < A / 2; ++n1) u[n1] = v[B * n1 + n2];
      rdft_half<A, DIR>(u);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = ctw<R, DIR>(u[k1], (n2 * k1) % R);
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      CP u[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) u[n2] = y[n2 * A + k1];
      rdft<B, DIR>(u);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
    }
  }
}

// X[n2] *= W_M^{DIR n2 k1} for n2 = 1 .. R2-1 from row k1 of the packed stage
// table: row[n2] = (c, c, s, s) with (c, s) = exp(-2 pi i n2 k1 / M). One
// 16-byte shared load serves both lines; n2 = 0 is the identity.
template <int R2, int DIR>
__device__ __forceinline__ void twiddle_row(CP* X, const float4* row) {
#pragma unroll
  for (int n2 = 1; n2 < R2; ++n2) {
    const float4 w = row[n2];
    const float2 cc = make_float2(w.x, w.y), ss = make_float2(w.z, w.w);
    const CP a = X[n2];
    if (DIR < 0) {   // (re c - im s, re s + im c)
      X[n2] = {psub(pmul(a.re, cc), pmul(a.im, ss)), pfma(a.re, ss, pmul(a.im, cc))};
    } else {         // (re c + im s, im c - re s)
      X[n2] = {pfma(a.im, ss, pmul(a.re, cc)), psub(pmul(a.im, cc), pmul(a.re, ss))};
    }
  }
}

// Global and shared layouts of a position of a line pair (lines a, b):
// AoS (the scalar engine's complex rows): float4 (re_a, im_a, re_b, im_b);
// split (the packed engine's spectral buffer): float4 (re_a, re_b, im_a, im_b).
__device__ __forceinline__ CP from_split(const float4 v) { return {make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
__device__ __forceinline__ float4 to_split(const CP& c) { return make_float4(c.re.x, c.re.y, c.im.x, c.im.y); }
__device__ __forceinline__ CP from_aos(const float4 v) { return {make_float2(v.x, v.z), make_float2(v.y, v.w)}; }
__device__ __forceinline__ float4 to_aos(const CP& c) { return make_float4(c.re.x, c.im.x, c.re.y, c.im.y); }

}  // namespace fft2p
}  // namespace gato
