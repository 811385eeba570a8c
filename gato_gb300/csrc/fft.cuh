// Shared-memory mixed-radix Stockham FFT engine (radices 2, 3, 4, 5, 7, 8).
//
// A CTA transforms L lines of length M at once. Shared memory holds two
// ping-pong buffers laid out position-major, buf[pos * LP + line] with
// LP = L + 1 (the pad keeps column loads of row-major data conflict-free).
// Consecutive threads take consecutive lines of one butterfly, so every
// stage's shared-memory access is a contiguous row segment.
//
// Stage s (radix R, Ns = product of earlier radices) follows the Stockham
// autosort formulation of Govindaraju et al., "High Performance Discrete
// Fourier Transforms on Graphics Processors" (SC'08): butterfly j reads
// in[j + r M/R], twiddles by exp(-+2 pi i r (j mod Ns)/(Ns R)), applies an
// R-point DFT and writes out[(j/Ns) Ns R + (j mod Ns) + r Ns].
#pragma once
#include "common.cuh"

namespace gato {

struct FftPlanDev {
  int M;
  int nst;
  int radix[16];
};

template <typename T2> struct CT;
template <> struct CT<float2> { using R = float; };
template <> struct CT<double2> { using R = double; };

template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) {
  a.x += b.x;
  a.y += b.y;
  return a;
}
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) {
  a.x -= b.x;
  a.y -= b.y;
  return a;
}
// multiply by dir * i  (dir = -1 forward, +1 inverse)
template <typename T2>
__device__ __forceinline__ T2 cmul_i(T2 a, int dir) {
  T2 r;
  if (dir < 0) {
    r.x = a.y;
    r.y = -a.x;
  } else {
    r.x = -a.y;
    r.y = a.x;
  }
  return r;
}

template <typename T2>
__device__ __forceinline__ void dft2(T2* v) {
  T2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <typename T2>
__device__ __forceinline__ void dft4(T2& v0, T2& v1, T2& v2, T2& v3, int dir) {
  T2 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = cmul_i(csub(v1, v3), dir);
  v0 = cadd(t0, t2);
  v2 = csub(t0, t2);
  v1 = cadd(t1, t3);
  v3 = csub(t1, t3);
}

template <typename T2>
__device__ __forceinline__ void dft8(T2* v, int dir) {
  using R = typename CT<T2>::R;
  const R s = (R)0.70710678118654752440;
  T2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  T2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4(e0, e1, e2, e3, dir);
  dft4(o0, o1, o2, o3, dir);
  // twiddles w8^q, w8 = exp(dir * 2 pi i / 8)
  T2 w1, w3;
  w1.x = s;
  w1.y = (R)dir * s;
  w3.x = -s;
  w3.y = (R)dir * s;
  o1 = cmul(o1, w1);
  o2 = cmul_i(o2, dir);
  o3 = cmul(o3, w3);
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}

// Direct odd-radix DFT with the exact cos/sin(2 pi k / R) constants.
template <int R>
__device__ __forceinline__ void odd_cs(int k, double& c, double& s) {
  if constexpr (R == 3) {
    c = k == 0 ? 1.0 : -0.5;
    s = k == 0 ? 0.0 : (k == 1 ? 0.86602540378443864676 : -0.86602540378443864676);
  } else if constexpr (R == 5) {
    switch (k) {
      case 0: c = 1.0; s = 0.0; break;
      case 1: c = 0.30901699437494742410; s = 0.95105651629515357212; break;
      case 2: c = -0.80901699437494742410; s = 0.58778525229247312917; break;
      case 3: c = -0.80901699437494742410; s = -0.58778525229247312917; break;
      default: c = 0.30901699437494742410; s = -0.95105651629515357212; break;
    }
  } else {
    switch (k) {
      case 0: c = 1.0; s = 0.0; break;
      case 1: c = 0.62348980185873353053; s = 0.78183148246802980871; break;
      case 2: c = -0.22252093395631440429; s = 0.97492791218182360702; break;
      case 3: c = -0.90096886790241912624; s = 0.43388373911755812048; break;
      case 4: c = -0.90096886790241912624; s = -0.43388373911755812048; break;
      case 5: c = -0.22252093395631440429; s = -0.97492791218182360702; break;
      default: c = 0.62348980185873353053; s = -0.78183148246802980871; break;
    }
  }
}

template <typename T2, int R>
__device__ __forceinline__ void dft_odd(T2* v, int dir) {
  using Rt = typename CT<T2>::R;
  T2 out[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    T2 acc = v[0];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      double cd, sd;
      odd_cs<R>((r * q) % R, cd, sd);
      const Rt c = (Rt)cd, sn = (Rt)dir * (Rt)sd;
      acc.x += v[r].x * c - v[r].y * sn;
      acc.y += v[r].x * sn + v[r].y * c;
    }
    out[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = out[q];
}

template <typename T2, int R>
__device__ __forceinline__ void dft_r(T2* v, int dir) {
  if constexpr (R == 2) dft2(v);
  else if constexpr (R == 4) dft4(v[0], v[1], v[2], v[3], dir);
  else if constexpr (R == 8) dft8(v, dir);
  else dft_odd<T2, R>(v, dir);
}

// One Stockham stage over L lines held in shared memory. `nin` < M marks
// positions >= nin of the input as zero (pruned zero-padded input).
template <typename T2, int R>
__device__ __forceinline__ void fft_stage(const T2* __restrict__ in, T2* __restrict__ out, int M,
                                          int Ns, int L, int LP, const T2* __restrict__ tw,
                                          int dir, int nin) {
  const int nbf = M / R;
  const int work = nbf * L;
  const int step = M / (Ns * R);
  for (int t = threadIdx.x; t < work; t += blockDim.x) {
    const int line = t % L;
    const int j = t / L;
    const int k = j % Ns;
    T2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int pos = j + r * nbf;
      if (pos < nin) v[r] = in[pos * LP + line];
      else v[r].x = v[r].y = 0;
    }
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        T2 w = tw[r * k * step];
        if (dir > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dft_r<T2, R>(v, dir);
    const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[(idxD + r * Ns) * LP + line] = v[r];
  }
}

// Full transform; returns the buffer holding the result. Begins and ends
// with __syncthreads().
template <typename T2>
__device__ T2* fft_lines(T2* A, T2* B, const FftPlanDev& pl, int L, int LP, const T2* tw, int dir,
                         int nin) {
  T2* in = A;
  T2* out = B;
  int Ns = 1;
  for (int s = 0; s < pl.nst; ++s) {
    __syncthreads();
    const int R = pl.radix[s];
    switch (R) {
      case 8: fft_stage<T2, 8>(in, out, pl.M, Ns, L, LP, tw, dir, nin); break;
      case 4: fft_stage<T2, 4>(in, out, pl.M, Ns, L, LP, tw, dir, nin); break;
      case 2: fft_stage<T2, 2>(in, out, pl.M, Ns, L, LP, tw, dir, nin); break;
      case 3: fft_stage<T2, 3>(in, out, pl.M, Ns, L, LP, tw, dir, nin); break;
      case 5: fft_stage<T2, 5>(in, out, pl.M, Ns, L, LP, tw, dir, nin); break;
      default: fft_stage<T2, 7>(in, out, pl.M, Ns, L, LP, tw, dir, nin); break;
    }
    nin = pl.M;
    Ns *= R;
    T2* t = in;
    in = out;
    out = t;
  }
  __syncthreads();
  return in;
}

// Host: factor M into the supported radices (largest first). Returns false
// if M has another prime factor.
inline bool fft_factor(int M, FftPlanDev& pl) {
  pl.M = M;
  pl.nst = 0;
  int m = M;
  const int rs[6] = {8, 4, 2, 3, 5, 7};
  for (int i = 0; i < 6; ++i) {
    while (m % rs[i] == 0 && pl.nst < 16) {
      pl.radix[pl.nst++] = rs[i];
      m /= rs[i];
    }
  }
  return m == 1 && M >= 2;
}

}  // namespace gato
