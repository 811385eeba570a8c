// Pair-solve pipeline kernels on the register-resident two-pass FFT engine
// (fft2.cuh), one instantiation per supported doubled-grid size M.
#pragma once
#include "fft2.cuh"
#include "poisson.cuh"

namespace gato {
namespace fast {

using namespace fft2;

template <typename T2>
__device__ __forceinline__ void load_tw(T2* tws, const T2* tw, int M) {
  for (int i = threadIdx.x; i < M; i += blockDim.x) tws[i] = tw[i];
}

// Strided-line passes (y forward, x forward * kernel * x inverse, y inverse).
template <typename T, int R1, int R2, int L, int MODE>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_cols(const typename Cplx<T>::type* in, typename Cplx<T>::type* out, ColGeom g,
           const typename Cplx<T>::type* tw, const T* ghat, int H) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, LP = L + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + M * LP;
  load_tw(tws, tw, M);
  const int outer = blockIdx.x, col0 = blockIdx.y * L, f = blockIdx.z;
  const int ncl = min(L, g.ncols - col0);
  const T2* src = in + f * g.in_fs + outer * g.in_os + col0;
  T2* dst = out + f * g.out_fs + outer * g.out_os + col0;
  const int t = threadIdx.x;
  const int line = t % L, q = t / L;   // q: n2 in stages 1/B, k1 in stages 2/A
  T2 X[R2];
  if (MODE != COL_INV) {
    if (q < R2)
      fwd_stage1<T2, R1, R2, true>(buf, LP, line, q, [&](int pos) {
        T2 v;
        if (line < ncl) v = src[pos * g.in_ps + line];
        else v.x = v.y = 0;
        return v;
      });
    __syncthreads();
    if (q < R1) fwd_stage2<T2, R1, R2>(buf, LP, line, q, tws, X);
  } else {
    __syncthreads();
    if (q < R1)
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        if (line < ncl) X[k2] = src[(q + R1 * k2) * g.in_ps + line];
        else X[k2].x = X[k2].y = 0;
      }
  }
  if (MODE == COL_FWD) {
    if (q < R1 && line < ncl)
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) dst[(q + R1 * k2) * g.out_ps + line] = X[k2];
    return;
  }
  if (MODE == COL_FMI && q < R1) {
    const int ky = outer, kyo = ky <= M - ky ? ky : M - ky;
    const int kz = col0 + line, kzo = kz <= M - kz ? kz : M - kz;
    const T* gp = ghat + (int64_t)kyo * H + kzo;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      const int kx = q + R1 * k2;
      const int kxo = kx <= M - kx ? kx : M - kx;
      const T gv = line < ncl ? gp[(int64_t)kxo * H * H] : (T)0;
      X[k2].x *= gv;
      X[k2].y *= gv;
    }
  }
  __syncthreads();   // stage-2 reads of buf are complete
  if (q < R1) inv_stageA<T2, R1, R2>(buf, LP, line, q, tws, X);
  __syncthreads();
  if (q < R2)
    inv_stageB<T2, R1, R2, true>(buf, LP, line, q, [&](int pos, T2 v) {
      if (line < ncl) dst[pos * g.out_ps + line] = v;
    });
}

// z forward with the pair-density prologue.
template <typename T, int R1, int R2, int L>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_rows_fwd(PassArgs args, int f0, typename Cplx<T>::type* S1, const typename Cplx<T>::type* tw) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, LP = L + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* stg = reinterpret_cast<T2*>(smraw);
  T2* buf = stg + M * LP;
  T2* tws = buf + M * LP;
  load_tw(tws, tw, M);
  const int p = blockIdx.y;
  const FieldDesc& fd = args.f[f0 + p];
  const int64_t row0 = (int64_t)blockIdx.x * L;
  const int64_t nrows = (int64_t)N * N;
  for (int i = threadIdx.x; i < L * N; i += blockDim.x) {
    const int line = i / N, z = i % N;
    const int64_t r = row0 + line;
    T2 v;
    v.x = v.y = 0;
    if (r < nrows) {
      const int64_t gi = r * N + z;
      v.x = dens<T>(fd.p[0], args.in, gi);
      if (fd.p[1].a >= 0) v.y = dens<T>(fd.p[1], args.in, gi);
    }
    stg[z * LP + line] = v;
  }
  __syncthreads();
  const int t = threadIdx.x, line = t % L, q = t / L;
  if (q < R2) fwd_stage1<T2, R1, R2, true>(buf, LP, line, q, [&](int pos) { return stg[pos * LP + line]; });
  __syncthreads();
  T2 X[R2];
  if (q < R1) {
    fwd_stage2<T2, R1, R2>(buf, LP, line, q, tws, X);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) stg[(q + R1 * k2) * LP + line] = X[k2];
  }
  __syncthreads();
  T2* dst = S1 + (int64_t)p * nrows * M;
  for (int i = threadIdx.x; i < L * M; i += blockDim.x) {
    const int ln = i / M, kz = i % M;
    const int64_t r = row0 + ln;
    if (r < nrows) dst[r * M + kz] = stg[kz * LP + ln];
  }
}

// z inverse over every field of the group, then the epilogue of poisson.cu.
template <typename T, int R1, int R2, int L, bool ENERGY>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_rows_inv(PassArgs args, int f0, int nfg, const typename Cplx<T>::type* S1,
               const typename Cplx<T>::type* tw, int accumulate, double* partials,
               int64_t slot_stride) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, LP = L + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sh[32];
  T2* stg = reinterpret_cast<T2*>(smraw);
  T2* buf = stg + M * LP;
  T2* tws = buf + M * LP;
  T* acc = reinterpret_cast<T*>(tws + M);
  load_tw(tws, tw, M);
  const int64_t row0 = (int64_t)blockIdx.x * L;
  const int64_t nrows = (int64_t)N * N;
  const int nout = args.nout;
  if (!ENERGY)
    for (int i = threadIdx.x; i < nout * L * N; i += blockDim.x) acc[i] = (T)0;
  Acc<T> e0, e1;
  const int t = threadIdx.x, line = t % L, q = t / L;
  for (int p = 0; p < nfg; ++p) {
    const FieldDesc& fd = args.f[f0 + p];
    const T2* src = S1 + (int64_t)p * nrows * M;
    __syncthreads();
    for (int i = threadIdx.x; i < L * M; i += blockDim.x) {
      const int ln = i / M, kz = i % M;
      const int64_t r = row0 + ln;
      T2 v;
      if (r < nrows) v = src[r * M + kz];
      else v.x = v.y = 0;
      stg[kz * LP + ln] = v;
    }
    __syncthreads();
    if (q < R1) {
      T2 X[R2];
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) X[k2] = stg[(q + R1 * k2) * LP + line];
      inv_stageA<T2, R1, R2>(buf, LP, line, q, tws, X);
    }
    __syncthreads();
    if (q < R2)
      inv_stageB<T2, R1, R2, true>(buf, LP, line, q, [&](int pos, T2 v) { stg[pos * LP + line] = v; });
    __syncthreads();
    for (int i = threadIdx.x; i < L * N; i += blockDim.x) {
      const int ln = i / N, z = i % N;
      const int64_t r = row0 + ln;
      if (r >= nrows) continue;
      const int64_t gi = r * N + z;
      const T2 J = stg[z * LP + ln];
#pragma unroll
      for (int qq = 0; qq < 2; ++qq) {
        const PartDesc& d = fd.p[qq];
        if (d.a < 0) continue;
        const T val = qq == 0 ? J.x : J.y;
        if (ENERGY) {
          const T de = dens<T>(d, args.in, gi);
          if (d.eslot == 0) e0.add_prod(de * (T)d.ew, val);
          else e1.add_prod(de * (T)d.ew, val);
        } else {
          for (int k = 0; k < d.nt; ++k) {
            T m = (T)d.coef[k];
            if (d.tc[k] >= 0) m *= reinterpret_cast<const T*>(args.in[d.tc[k]])[gi];
            acc[(d.to[k] * L + ln) * N + z] += m * val;
          }
        }
      }
    }
  }
  if (ENERGY) {
    const double s0 = block_sum(e0.value(), sh);
    const double s1 = block_sum(e1.value(), sh);
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = s0;
      partials[slot_stride + blockIdx.x] = s1;
    }
  } else {
    __syncthreads();
    for (int o = 0; o < nout; ++o) {
      T* dst = reinterpret_cast<T*>(args.out[o]);
      for (int i = threadIdx.x; i < L * N; i += blockDim.x) {
        const int ln = i / N, z = i % N;
        const int64_t r = row0 + ln;
        if (r >= nrows) continue;
        const int64_t gi = r * N + z;
        const T v = acc[(o * L + ln) * N + z];
        dst[gi] = accumulate ? dst[gi] + v : v;
      }
    }
  }
}

template <typename K>
inline int smem_attr(K k, size_t bytes) {
  GATO_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return GATO_OK;
}

// Launchers for one shape.
template <typename T, int R1, int R2, int L>
struct Launch {
  using T2 = typename Cplx<T>::type;
  static constexpr int M = R1 * R2, N = M / 2, NT = L * Shape<R1, R2>::RMAX;
  static size_t sm_cols() { return (size_t)(M * (L + 1) + M) * sizeof(T2); }
  static size_t sm_rows(int nout) {
    return (size_t)(2 * M * (L + 1) + M) * sizeof(T2) + (size_t)nout * L * N * sizeof(T);
  }
  static int cols(int mode, const T2* in, T2* out, const ColGeom& g, int outer, int nf, const T2* tw,
                  const T* ghat, int H, cudaStream_t s) {
    dim3 grid(outer, (g.ncols + L - 1) / L, nf);
    const size_t sm = sm_cols();
    if (mode == COL_FWD) {
      GATO_TRY(smem_attr(k_cols<T, R1, R2, L, COL_FWD>, sm));
      k_cols<T, R1, R2, L, COL_FWD><<<grid, NT, sm, s>>>(in, out, g, tw, ghat, H);
    } else if (mode == COL_INV) {
      GATO_TRY(smem_attr(k_cols<T, R1, R2, L, COL_INV>, sm));
      k_cols<T, R1, R2, L, COL_INV><<<grid, NT, sm, s>>>(in, out, g, tw, ghat, H);
    } else {
      GATO_TRY(smem_attr(k_cols<T, R1, R2, L, COL_FMI>, sm));
      k_cols<T, R1, R2, L, COL_FMI><<<grid, NT, sm, s>>>(in, out, g, tw, ghat, H);
    }
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  static int rows_fwd(const PassArgs& a, int f0, int nfg, T2* S1, const T2* tw, cudaStream_t s) {
    const size_t sm = sm_rows(0);
    GATO_TRY(smem_attr(k_rows_fwd<T, R1, R2, L>, sm));
    const int64_t nrows = (int64_t)N * N;
    k_rows_fwd<T, R1, R2, L><<<dim3((unsigned)((nrows + L - 1) / L), nfg), NT, sm, s>>>(a, f0, S1, tw);
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  static int rows_inv(const PassArgs& a, int f0, int nfg, const T2* S1, const T2* tw, int accumulate,
                      bool energy, double* partials, int64_t slot_stride, cudaStream_t s) {
    const size_t sm = sm_rows(energy ? 0 : a.nout);
    const unsigned nblk = (unsigned)(((int64_t)N * N + L - 1) / L);
    if (energy) {
      GATO_TRY(smem_attr(k_rows_inv<T, R1, R2, L, true>, sm));
      k_rows_inv<T, R1, R2, L, true><<<nblk, NT, sm, s>>>(a, f0, nfg, S1, tw, accumulate, partials,
                                                          slot_stride);
    } else {
      GATO_TRY(smem_attr(k_rows_inv<T, R1, R2, L, false>, sm));
      k_rows_inv<T, R1, R2, L, false><<<nblk, NT, sm, s>>>(a, f0, nfg, S1, tw, accumulate, partials,
                                                           slot_stride);
    }
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
};

}  // namespace fast
}  // namespace gato
