// FFT-Poisson Hartree solve and pairwise exchange (solvers/poisson.py:29-92,
// scf.py:66-85) on the Hockney doubled grid M = 2N.
//
// Two real densities ride in one complex field (re + i im): the kernel
// spectrum is real and even, so the product with it keeps the two parts
// apart and the inverse transform returns J[re] + i J[im]. Per batch of
// fields the pipeline is five launches, each a set of batched 1-D
// transforms staged in shared memory:
//   rows_fwd : form the pair densities on the fly, FFT along z (N nonzero
//              of M), write S1[f][x<N][y<N][kz<M]
//   cols FWD : FFT along y (N nonzero of M)  -> S2[f][x<N][ky<M][kz<M]
//   cols FMI : FFT along x (N nonzero), multiply by the kernel octant,
//              inverse FFT along x keeping x < N (in place in S2)
//   cols INV : inverse FFT along y keeping y < N -> S1
//   rows_inv : inverse FFT along z keeping z < N, then the epilogue:
//              accumulate coef * u * J into outputs (exchange, Hartree) or
//              reduce weighted density * J (energies).
// The kernel spectrum is computed once per plan in FP64 with the same
// engine and stored as its (M/2+1)^3 octant (it is even in every axis).
#include <algorithm>
#include <type_traits>
#include <cmath>
#include <vector>

#include "fft2.cuh"
#include "poisson.cuh"

namespace gato {

namespace {

constexpr int kFftThreads = 256;

template <typename T2>
inline size_t fft_smem(int M, int L) {
  return (size_t)2 * M * (L + 1) * sizeof(T2) + (size_t)M * sizeof(T2);
}

template <typename T2>
int pick_L(int M, size_t extra_per_line, int Lmax) {
  for (int L = Lmax; L >= 1; L >>= 1)
    if (fft_smem<T2>(M, L) + extra_per_line * L <= 112 * 1024) return L;
  return 1;
}

template <typename T2>
__device__ __forceinline__ void load_twiddles(T2* tw_s, const T2* tw, int M) {
  for (int i = threadIdx.x; i < M; i += blockDim.x) tw_s[i] = tw[i];
}

// ---- kernel spectrum (FP64) ----------------------------------------------------

// Rows of the softened kernel G (poisson.py:29-44), FFT along z.
__global__ void k_ghat_rows(double2* X, FftPlanDev pl, const double2* tw, int N, double h,
                            double eps, int L) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int M = pl.M, LP = L + 1;
  double2* A = reinterpret_cast<double2*>(sm);
  double2* B = A + M * LP;
  double2* tws = B + M * LP;
  load_twiddles(tws, tw, M);
  const int64_t row0 = (int64_t)blockIdx.x * L;
  for (int t = threadIdx.x; t < L * M; t += blockDim.x) {
    const int line = t / M, z = t % M;
    const int64_t r = row0 + line;
    const int x = (int)(r / M), y = (int)(r % M);
    auto disp = [&](int i) { return i < N ? i * h : (i - M) * h; };
    const double dx = disp(x), dy = disp(y), dz = disp(z);
    double2 v;
    v.x = (r < (int64_t)M * M) ? 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps * eps) : 0.0;
    v.y = 0.0;
    A[z * LP + line] = v;
  }
  double2* res = fft_lines(A, B, pl, L, LP, tws, -1, M);
  for (int t = threadIdx.x; t < L * M; t += blockDim.x) {
    const int line = t / M, kz = t % M;
    const int64_t r = row0 + line;
    if (r < (int64_t)M * M) X[r * M + kz] = res[kz * LP + line];
  }
}

template <typename T>
__global__ void k_ghat_extract(const double2* X, T* ghat, int M, int H, double scale) {
  const int64_t n = (int64_t)H * H * H;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % H);
    const int b = (int)((i / H) % H);
    const int a = (int)(i / ((int64_t)H * H));
    ghat[i] = (T)(X[((int64_t)a * M + b) * M + c].x * scale);
  }
}

// The packed FP32 engine's kernel spectrum: the octant unfolded along z,
// ghat2[(kxo H + kyo) M + kz] = ghat[(kxo H + kyo) H + min(kz, M - kz)], so a
// column pair (kz, kz + 1) reads one aligned float2.
__global__ void k_ghat_unfold_z(const float* ghat, float* ghat2, int M, int H) {
  const int64_t n = (int64_t)H * H * M;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(i % M);
    const int64_t ab = i / M;
    ghat2[i] = ghat[ab * H + (kz <= M - kz ? kz : M - kz)];
  }
}

// ---- batched strided-line transforms ------------------------------------------

template <typename T2, int MODE>
__global__ void __launch_bounds__(kFftThreads)
    k_cols(const T2* in, T2* out, ColGeom g, FftPlanDev pl, const T2* tw,
           const typename CT<T2>::R* ghat, int H, int L) {
  using T = typename CT<T2>::R;
  extern __shared__ __align__(16) unsigned char sm[];
  const int M = pl.M, LP = L + 1;
  T2* A = reinterpret_cast<T2*>(sm);
  T2* B = A + M * LP;
  T2* tws = B + M * LP;
  load_twiddles(tws, tw, M);
  const int outer = blockIdx.x;
  const int col0 = blockIdx.y * L;
  const int f = blockIdx.z;
  const int ncl = min(L, g.ncols - col0);
  const T2* src = in + f * g.in_fs + outer * g.in_os + col0;
  for (int t = threadIdx.x; t < g.nin * L; t += blockDim.x) {
    const int line = t % L, pos = t / L;
    T2 v;
    if (line < ncl) v = src[pos * g.in_ps + line];
    else v.x = v.y = 0;
    A[pos * LP + line] = v;
  }
  T2* res = fft_lines(A, B, pl, L, LP, tws, MODE == COL_INV ? +1 : -1, g.nin);
  if (MODE == COL_FMI) {
    const int ky = outer, kyo = ky <= M - ky ? ky : M - ky;
    for (int t = threadIdx.x; t < M * L; t += blockDim.x) {
      const int line = t % L, kx = t / L;
      const int kz = col0 + line;
      const int kxo = kx <= M - kx ? kx : M - kx;
      const int kzo = kz <= M - kz ? kz : M - kz;
      const T gv = (line < ncl) ? ghat[((int64_t)kxo * H + kyo) * H + kzo] : (T)0;
      T2 v = res[kx * LP + line];
      v.x *= gv;
      v.y *= gv;
      res[kx * LP + line] = v;
    }
    res = fft_lines(res, res == A ? B : A, pl, L, LP, tws, +1, M);
  }
  T2* dst = out + f * g.out_fs + outer * g.out_os + col0;
  for (int t = threadIdx.x; t < g.nout * L; t += blockDim.x) {
    const int line = t % L, pos = t / L;
    if (line < ncl) dst[pos * g.out_ps + line] = res[pos * LP + line];
  }
}

// Forward z rows with the pair-density prologue.
template <typename T>
__global__ void __launch_bounds__(kFftThreads)
    k_rows_fwd(PassArgs args, int f0, typename Cplx<T>::type* S1, FftPlanDev pl,
               const typename Cplx<T>::type* tw, int N, int L) {
  using T2 = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char sm[];
  const int M = pl.M, LP = L + 1;
  T2* A = reinterpret_cast<T2*>(sm);
  T2* B = A + M * LP;
  T2* tws = B + M * LP;
  load_twiddles(tws, tw, M);
  const int p = blockIdx.y;
  const FieldDesc& fd = args.f[f0 + p];
  const int64_t row0 = (int64_t)blockIdx.x * L;
  const int64_t nrows = (int64_t)N * N;
  for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
    const int line = t / N, z = t % N;
    const int64_t r = row0 + line;
    T2 v;
    v.x = v.y = 0;
    if (r < nrows) {
      const int64_t gi = r * N + z;
      v.x = dens<T>(fd.p[0], args.in, gi);
      if (fd.p[1].a >= 0) v.y = dens<T>(fd.p[1], args.in, gi);
    }
    A[z * LP + line] = v;
  }
  T2* res = fft_lines(A, B, pl, L, LP, tws, -1, N);
  T2* dst = S1 + (int64_t)p * nrows * M;
  for (int t = threadIdx.x; t < L * M; t += blockDim.x) {
    const int line = t / M, kz = t % M;
    const int64_t r = row0 + line;
    if (r < nrows) dst[r * M + kz] = res[kz * LP + line];
  }
}

// Inverse z rows over every field of the group, with the epilogue.
template <typename T, bool ENERGY>
__global__ void __launch_bounds__(kFftThreads)
    k_rows_inv(PassArgs args, int f0, int nfg, const typename Cplx<T>::type* S1, FftPlanDev pl,
               const typename Cplx<T>::type* tw, int N, int L, int accumulate,
               double* partials, int64_t slot_stride) {
  using T2 = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double sh[32];
  const int M = pl.M, LP = L + 1;
  T2* A = reinterpret_cast<T2*>(sm);
  T2* B = A + M * LP;
  T2* tws = B + M * LP;
  T* acc = reinterpret_cast<T*>(tws + M);   // nout x L x N
  load_twiddles(tws, tw, M);
  const int64_t row0 = (int64_t)blockIdx.x * L;
  const int64_t nrows = (int64_t)N * N;
  const int nout = args.nout;
  if (!ENERGY)
    for (int t = threadIdx.x; t < nout * L * N; t += blockDim.x) acc[t] = (T)0;
  Acc<T> e0, e1;
  for (int p = 0; p < nfg; ++p) {
    const FieldDesc& fd = args.f[f0 + p];
    const T2* src = S1 + (int64_t)p * nrows * M;
    __syncthreads();
    for (int t = threadIdx.x; t < L * M; t += blockDim.x) {
      const int line = t / M, kz = t % M;
      const int64_t r = row0 + line;
      T2 v;
      if (r < nrows) v = src[r * M + kz];
      else v.x = v.y = 0;
      A[kz * LP + line] = v;
    }
    T2* res = fft_lines(A, B, pl, L, LP, tws, +1, M);
    for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
      const int line = t / N, z = t % N;
      const int64_t r = row0 + line;
      if (r >= nrows) continue;
      const int64_t gi = r * N + z;
      const T2 J = res[z * LP + line];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const PartDesc& d = fd.p[q];
        if (d.a < 0) continue;
        const T val = q == 0 ? J.x : J.y;
        if (ENERGY) {
          const T de = dens<T>(d, args.in, gi);
          const double w = d.ew;
          if (d.eslot == 0) e0.add_prod(de * (T)w, val);
          else e1.add_prod(de * (T)w, val);
        } else {
          for (int k = 0; k < d.nt; ++k) {
            T m = (T)d.coef[k];
            if (d.tc[k] >= 0) m *= reinterpret_cast<const T*>(args.in[d.tc[k]])[gi];
            acc[(d.to[k] * L + line) * N + z] += m * val;
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
      for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
        const int line = t / N, z = t % N;
        const int64_t r = row0 + line;
        if (r >= nrows) continue;
        const int64_t gi = r * N + z;
        const T v = acc[(o * L + line) * N + z];
        dst[gi] = accumulate ? dst[gi] + v : v;
      }
    }
  }
}

template <typename KernelT>
int set_smem(KernelT k, size_t bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(k), bytes);
}

template <typename T2>
int launch_cols(int mode, const T2* in, T2* out, const ColGeom& g, int outer, int nf,
                const FftPlanDev& fp, const T2* tw, const typename CT<T2>::R* ghat, int H,
                cudaStream_t s) {
  const int L = pick_L<T2>(fp.M, 0, sizeof(T2) == 8 ? 16 : 8);
  const size_t sm = fft_smem<T2>(fp.M, L);
  dim3 grid(outer, (g.ncols + L - 1) / L, nf);
  if (mode == COL_FWD) {
    GATO_TRY(set_smem(k_cols<T2, COL_FWD>, sm));
    k_cols<T2, COL_FWD><<<grid, kFftThreads, sm, s>>>(in, out, g, fp, tw, ghat, H, L);
  } else if (mode == COL_INV) {
    GATO_TRY(set_smem(k_cols<T2, COL_INV>, sm));
    k_cols<T2, COL_INV><<<grid, kFftThreads, sm, s>>>(in, out, g, fp, tw, ghat, H, L);
  } else {
    GATO_TRY(set_smem(k_cols<T2, COL_FMI>, sm));
    k_cols<T2, COL_FMI><<<grid, kFftThreads, sm, s>>>(in, out, g, fp, tw, ghat, H, L);
  }
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

template <typename T>
int run_typed(PoissonPlan& pl, const PassArgs& args, int epi, bool accumulate, double* energy_dev,
              cudaStream_t s, cudaEvent_t join) {
  using T2 = typename Cplx<T>::type;
  const int N = pl.N, M = pl.M;
  const int64_t nrows = (int64_t)N * N;
  const T2* tw = (const T2*)pl.tw;
  const T2* tw2 = (const T2*)pl.tw2;   // the register engine's per-row stage twiddles
  T2* S1 = (T2*)pl.S1;
  T2* S2 = (T2*)pl.S2;
  const int Lf = pl.engine != 1 ? fast::rows_L<T>(M) : 0;   // register engine, 0: generic
  // FP32 register engine: the column passes run packed (two lines per thread) where M has an
  // instantiation, unless engine 4 asks for the scalar ones; the FP64 spectral energy pass never
  // meets an FP32 plan
  const bool packed = sizeof(T) == 4 && Lf > 0 && pl.tw4 && pl.engine != 4;
  const int Lr = pick_L<T2>(M, 0, sizeof(T) == 4 ? 16 : 8);
  const int Li = pick_L<T2>(M, (size_t)args.nout * N * sizeof(T), sizeof(T) == 4 ? 16 : 8);
  const size_t sm_r = fft_smem<T2>(M, Lr);
  const size_t sm_i = fft_smem<T2>(M, Li) + (size_t)args.nout * Li * N * sizeof(T);
  const int Linv = Lf > 0 ? Lf : Li;
  const int nblk_i = (int)((nrows + Linv - 1) / Linv);
  const int group = pl.group > 0 ? std::min(pl.group, pl.max_fields) : pl.max_fields;
  const int ngroups = (args.nf + group - 1) / group;
  // FP64 energies on the register engine take the spectral (Parseval) pass
  // when both parts of every field carry one weight and one slot: x forward
  // and the kernel-weighted power, no x, y or z inverse.
  bool fe = epi == EPI_ENERGY && poisson_fe_supported(pl);
  const int64_t fe_nb = fe ? (int64_t)M * ((M + Lf - 1) / Lf) : 0;   // x-pass CTAs per field
  FeArgs fa;
  if (fe) {
    for (int f = 0; f < args.nf && fe; ++f) {
      const PartDesc& p0 = args.f[f].p[0];
      const PartDesc& p1 = args.f[f].p[1];
      const PartDesc& pw = p0.a >= 0 ? p0 : p1;
      fe = (p0.a < 0 || p1.a < 0 || (p0.ew == p1.ew && p0.eslot == p1.eslot)) && pw.eslot >= 0 &&
           pw.eslot <= 1;
      fa.w[f] = pw.a >= 0 ? pw.ew : 0.0;
      fa.slot[f] = pw.eslot;
    }
    fe = fe && 2 * args.nf * fe_nb <= pl.npart_cap;
    fa.partials = pl.partials;
    fa.slot_stride = args.nf * fe_nb;
  }
  if (epi == EPI_ENERGY && !fe && (int64_t)ngroups * 2 * nblk_i > pl.npart_cap)
    return fail(GATO_EUNSUPPORTED, "poisson: energy partials exceed plan capacity");
  if (Lf == 0) {
    GATO_TRY(set_smem(k_rows_fwd<T>, sm_r));
    if (epi == EPI_ENERGY) GATO_TRY(set_smem(k_rows_inv<T, true>, sm_i));
    else GATO_TRY(set_smem(k_rows_inv<T, false>, sm_i));
  }
  ColGeom gy{nrows * M, (int64_t)N * M * M, (int64_t)N * M, (int64_t)M * M, M, M, M, N, M};
  ColGeom gx{(int64_t)N * M * M, (int64_t)N * M * M, M, M, (int64_t)M * M, (int64_t)M * M, M, N, N};
  ColGeom gyi{(int64_t)N * M * M, nrows * M, (int64_t)M * M, (int64_t)N * M, M, M, M, M, N};
  for (int g = 0; g < ngroups; ++g) {
    const int f0 = g * group;
    const int nfg = std::min(group, args.nf - f0);
    const bool acc_here = accumulate || g > 0;
    double* part = pl.partials + (int64_t)g * nblk_i;
    const int64_t sstride = (int64_t)ngroups * nblk_i;
    if (Lf > 0) {
      // register-resident two-pass engine
      // engine 0: multi-field z forward from two fields, 2: never, 3: from three
      GATO_TRY(fast::rows_fwd<T>(M, args, f0, nfg, S1, tw2, pl.engine == 2 ? 0 : (pl.engine == 3 ? 1 : (pl.engine == 4 ? 3 : 2)), s));
      if (packed) {
        // FP32 column passes on the packed two-line engine (S2 in the split pair layout)
        GATO_TRY(fast::packed_cols(M, COL_FWD, (const float2*)S1, (float2*)S2, gy, N, nfg,
                                   (const float4*)pl.tw4, nullptr, pl.H, s));
        GATO_TRY(fast::packed_cols(M, COL_FMI, (const float2*)S2, (float2*)S2, gx, M, nfg,
                                   (const float4*)pl.tw4, (const float*)pl.ghat2, pl.H, s));
        GATO_TRY(fast::packed_cols(M, COL_INV, (const float2*)S2, (float2*)S1, gyi, N, nfg,
                                   (const float4*)pl.tw4, nullptr, pl.H, s));
      } else {
      GATO_TRY(fast::cols<T>(M, COL_FWD, S1, S2, gy, N, nfg, tw2, nullptr, pl.H, s));
      if constexpr (sizeof(T) == 8) {
        if (fe) {
          fa.f0 = f0;
          GATO_TRY(fast::cols_fe<T>(M, S2, gx, M, nfg, tw2, (const T*)pl.ghat, pl.H, fa, s));
          continue;
        }
      }
      GATO_TRY(fast::cols<T>(M, COL_FMI, S2, S2, gx, M, nfg, tw2, (const T*)pl.ghat, pl.H, s));
      GATO_TRY(fast::cols<T>(M, COL_INV, S2, S1, gyi, N, nfg, tw2, nullptr, pl.H, s));
      }
      if (join && g == 0 && epi == EPI_ACC) GATO_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
      if (epi == EPI_J)
        GATO_TRY(fast::rows_inv_j<T>(M, args, f0, nfg, S1, tw2, s));
      else
        GATO_TRY(fast::rows_inv<T>(M, args, f0, nfg, S1, tw2, acc_here ? 1 : 0, epi == EPI_ENERGY, part,
                                   sstride, s));
      continue;
    }
    if (epi == EPI_J) return fail(GATO_EUNSUPPORTED, "poisson: J output needs the register engine");
    // 1. z forward with the pair-density prologue
    k_rows_fwd<T><<<dim3((unsigned)((nrows + Lr - 1) / Lr), nfg), kFftThreads, sm_r, s>>>(
        args, f0, S1, pl.fp, tw, N, Lr);
    GATO_LAUNCH_TRY();
    // 2. y forward: S1[f][x][y<N][kz] -> S2[f][x][ky][kz]
    GATO_TRY(launch_cols<T2>(COL_FWD, S1, S2, gy, N, nfg, pl.fp, tw, nullptr, pl.H, s));
    // 3. x forward, kernel multiply, x inverse (in place)
    GATO_TRY(launch_cols<T2>(COL_FMI, S2, S2, gx, M, nfg, pl.fp, tw, (const T*)pl.ghat, pl.H, s));
    // 4. y inverse: S2[f][x][ky][kz] -> S1[f][x][y<N][kz]
    GATO_TRY(launch_cols<T2>(COL_INV, S2, S1, gyi, N, nfg, pl.fp, tw, nullptr, pl.H, s));
    // 5. z inverse + epilogue
    if (join && g == 0 && epi == EPI_ACC) GATO_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
    if (epi == EPI_ENERGY)
      k_rows_inv<T, true><<<nblk_i, kFftThreads, sm_i, s>>>(args, f0, nfg, S1, pl.fp, tw, N, Li, 0,
                                                            part, sstride);
    else
      k_rows_inv<T, false><<<nblk_i, kFftThreads, sm_i, s>>>(args, f0, nfg, S1, pl.fp, tw, N, Li,
                                                             acc_here ? 1 : 0, nullptr, 0);
    GATO_LAUNCH_TRY();
  }
  if (epi == EPI_ENERGY) {
    // partials laid out [slot][group][row block], or [slot][field][x-pass block]
    const int64_t nparts = fe ? args.nf * fe_nb : (int64_t)ngroups * nblk_i;
    GATO_TRY(finalize_sums(pl.partials, 2, (int)nparts, pl.dV, energy_dev, s));
  }
  return GATO_OK;
}

}  // namespace

int poisson_run(PoissonPlan& pl, const PassArgs& args, int epi, bool accumulate,
                double* energy_dev, cudaStream_t s, cudaEvent_t join) {
  if (args.nf <= 0) {
    if (join) GATO_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
    return GATO_OK;
  }
  if (args.nf > kMaxFields) return fail(GATO_EBADARG, "poisson: too many fields (%d)", args.nf);
  if (pl.dtype == GATO_F64) return run_typed<double>(pl, args, epi, accumulate, energy_dev, s, join);
  return run_typed<float>(pl, args, epi, accumulate, energy_dev, s, join);
}

static int plan_create(int dtype, int N, double h, double eps, int max_fields, PoissonPlan& pl,
                       cudaStream_t s) {
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  if (N < 1 || h <= 0 || !(eps >= 0) || max_fields < 1)
    return fail(GATO_EBADARG, "poisson plan: bad arguments (N=%d h=%g eps=%g)", N, h, eps);
  const int M = 2 * N;
  if (!fft_factor(M, pl.fp))
    return fail(GATO_EUNSUPPORTED, "poisson plan: M=2N=%d must factor into 2,3,5,7", M);
  pl.dtype = dtype;
  pl.N = N;
  pl.M = M;
  pl.H = M / 2 + 1;
  pl.h = h;
  pl.eps = eps;
  pl.dV = h * h * h;
  pl.max_fields = max_fields;
  const size_t ts = dtype == GATO_F64 ? sizeof(double) : sizeof(float);
  // twiddles of both precisions (the spectrum build is FP64)
  std::vector<double2> tw64(M);
  std::vector<float2> tw32(M);
  for (int k = 0; k < M; ++k) {
    const double a = 2.0 * 3.14159265358979323846 * (double)k / (double)M;
    tw64[k] = make_double2(cos(a), -sin(a));
    tw32[k] = make_float2((float)tw64[k].x, (float)tw64[k].y);
  }
  GATO_CUDA_TRY(cudaMalloc(&pl.tw, (size_t)M * 2 * ts));
  // uploads go on s: a blocking cudaMemcpy from pageable memory may return before its DMA lands
  // and is not ordered against a non-blocking s, whose kernels read these tables next (a pageable
  // cudaMemcpyAsync returns once the host data is staged, so the vectors may go out of scope)
  GATO_CUDA_TRY(cudaMemcpyAsync(pl.tw, dtype == GATO_F64 ? (void*)tw64.data() : (void*)tw32.data(),
                                (size_t)M * 2 * ts, cudaMemcpyHostToDevice, s));
  if (const int R2 = fast::shape_r2(M)) {
    // the register engine's stage twiddles: row k1 holds exp(-2 pi i n2 k1 / M)
    // for n2 < R2, rows padded to the stride the kernels read them with
    const int R1 = M / R2;
    const int S = fft2::tw_row_stride(dtype == GATO_F32, R2);
    std::vector<double2> t64((size_t)R1 * S, make_double2(0.0, 0.0));
    std::vector<float2> t32((size_t)R1 * S, make_float2(0.f, 0.f));
    for (int k1 = 0; k1 < R1; ++k1)
      for (int n2 = 0; n2 < R2; ++n2) {
        const double2 w = tw64[(size_t)n2 * k1];   // n2 k1 < M
        t64[(size_t)k1 * S + n2] = w;
        t32[(size_t)k1 * S + n2] = make_float2((float)w.x, (float)w.y);
      }
    const size_t bytes = (size_t)R1 * S * 2 * ts;
    GATO_CUDA_TRY(cudaMalloc(&pl.tw2, bytes));
    GATO_CUDA_TRY(cudaMemcpyAsync(pl.tw2, dtype == GATO_F64 ? (void*)t64.data() : (void*)t32.data(), bytes,
                                  cudaMemcpyHostToDevice, s));
  }
  if (const int R2 = dtype == GATO_F32 ? fast::packed_r2(M) : 0) {
    // packed stage twiddles: entry k1 R2 + n2 = (c, c, s, s), (c, s) = exp(-2 pi i n2 k1 / M)
    const int R1 = M / R2;
    std::vector<float4> t4((size_t)R1 * R2);
    for (int k1 = 0; k1 < R1; ++k1)
      for (int n2 = 0; n2 < R2; ++n2) {
        const float c = (float)tw64[(size_t)n2 * k1].x, sn = (float)tw64[(size_t)n2 * k1].y;
        t4[(size_t)k1 * R2 + n2] = make_float4(c, c, sn, sn);
      }
    GATO_CUDA_TRY(cudaMalloc(&pl.tw4, t4.size() * sizeof(float4)));
    GATO_CUDA_TRY(cudaMemcpyAsync(pl.tw4, t4.data(), t4.size() * sizeof(float4), cudaMemcpyHostToDevice, s));
  }
  double2* tw_d = nullptr;
  GATO_CUDA_TRY(cudaMalloc(&tw_d, (size_t)M * sizeof(double2)));
  GATO_CUDA_TRY(cudaMemcpyAsync(tw_d, tw64.data(), (size_t)M * sizeof(double2), cudaMemcpyHostToDevice, s));
  // kernel spectrum in FP64 on an M^3 complex scratch
  double2* X = nullptr;
  const size_t xbytes = (size_t)M * M * M * sizeof(double2);
  GATO_CUDA_TRY(cudaMalloc(&X, xbytes));
  const int L = pick_L<double2>(M, 0, 8);
  const size_t sm = fft_smem<double2>(M, L);
  GATO_TRY(set_smem(k_ghat_rows, sm));
  const int64_t rows = (int64_t)M * M;
  k_ghat_rows<<<(unsigned)((rows + L - 1) / L), kFftThreads, sm, s>>>(X, pl.fp, tw_d, N, h, eps, L);
  GATO_LAUNCH_TRY();
  ColGeom gy{0, 0, (int64_t)M * M, (int64_t)M * M, M, M, M, M, M};
  GATO_TRY(launch_cols<double2>(COL_FWD, X, X, gy, M, 1, pl.fp, tw_d, nullptr, pl.H, s));
  ColGeom gx{0, 0, M, M, (int64_t)M * M, (int64_t)M * M, M, M, M};
  GATO_TRY(launch_cols<double2>(COL_FWD, X, X, gx, M, 1, pl.fp, tw_d, nullptr, pl.H, s));
  const int64_t oct = (int64_t)pl.H * pl.H * pl.H;
  GATO_CUDA_TRY(cudaMalloc(&pl.ghat, oct * ts));
  const double scale = pl.dV / ((double)M * M * M);
  if (dtype == GATO_F64)
    k_ghat_extract<double><<<grid_for(oct, 256), 256, 0, s>>>(X, (double*)pl.ghat, M, pl.H, scale);
  else
    k_ghat_extract<float><<<grid_for(oct, 256), 256, 0, s>>>(X, (float*)pl.ghat, M, pl.H, scale);
  GATO_LAUNCH_TRY();
  if (pl.tw4) {
    const int64_t n2 = (int64_t)pl.H * pl.H * M;
    GATO_CUDA_TRY(cudaMalloc(&pl.ghat2, n2 * sizeof(float)));
    k_ghat_unfold_z<<<grid_for(n2, 256), 256, 0, s>>>((const float*)pl.ghat, (float*)pl.ghat2, M, pl.H);
    GATO_LAUNCH_TRY();
  }
  GATO_CUDA_TRY(cudaStreamSynchronize(s));
  cudaFree(X);
  cudaFree(tw_d);
  // spectral buffers
  const size_t cs = 2 * ts;
  GATO_CUDA_TRY(cudaMalloc(&pl.S1, (size_t)max_fields * N * N * M * cs));
  GATO_CUDA_TRY(cudaMalloc(&pl.S2, (size_t)max_fields * N * M * M * cs));
  // energy partials: 2 slots x (groups of a 40-field call) x row blocks (L >= 1);
  // the FP64 spectral pass needs 2 slots x fields x x-pass CTAs (room for 2 max_fields)
  pl.npart_cap = 2 * ((kMaxFields + max_fields - 1) / max_fields) * N * N;
  const int Lc = dtype == GATO_F64 ? fast::rows_L<double>(M) : 0;
  if (Lc > 0) pl.npart_cap = std::max(pl.npart_cap, 2 * 2 * max_fields * M * ((M + Lc - 1) / Lc));
  GATO_CUDA_TRY(cudaMalloc(&pl.partials, (size_t)pl.npart_cap * sizeof(double)));
  return GATO_OK;
}

static void plan_free(PoissonPlan& pl) {
  free_after_pending({pl.ghat, pl.tw, pl.tw2, pl.tw4, pl.ghat2, pl.S1, pl.S2, pl.partials});
  pl = PoissonPlan{};
}

}  // namespace gato

using namespace gato;

extern "C" int gato_poisson_create(int dtype, int N, double h, double eps, int max_fields,
                                   gato_poisson_t* out, void* stream) {
  if (!out) return fail(GATO_EBADARG, "gato_poisson_create: out is NULL");
  auto* p = new gato_poisson_plan();
  int st = plan_create(dtype, N, h, eps, max_fields, p->p, as_stream(stream));
  if (st != GATO_OK) {
    plan_free(p->p);
    delete p;
    return st;
  }
  *out = p;
  return GATO_OK;
}

extern "C" int gato_poisson_destroy(gato_poisson_t plan) {
  if (!plan) return GATO_OK;
  plan_free(plan->p);
  delete plan;
  return GATO_OK;
}

extern "C" int gato_hartree_potential(gato_poisson_t plan, const void* rho, void* J, void* stream) {
  if (!plan || !rho || !J) return fail(GATO_EBADARG, "gato_hartree_potential: bad arguments");
  PassArgs a;
  a.in[0] = rho;
  a.out[0] = J;
  a.nout = 1;
  a.nf = 1;
  a.f[0].p[0].a = 0;
  a.f[0].p[0].nt = 1;
  a.f[0].p[0].to[0] = 0;
  a.f[0].p[0].coef[0] = 1.f;
  return poisson_run(plan->p, a, EPI_ACC, false, nullptr, as_stream(stream));
}

extern "C" int gato_hartree_energy(gato_poisson_t plan, const void* rho, double* E_dev,
                                   void* stream) {
  if (!plan || !rho || !E_dev) return fail(GATO_EBADARG, "gato_hartree_energy: bad arguments");
  PassArgs a;
  a.in[0] = rho;
  a.nf = 1;
  a.f[0].p[0].a = 0;
  a.f[0].p[0].ew = 0.5;
  a.f[0].p[0].eslot = 0;
  double* tmp = (double*)stream_scratch(as_stream(stream), 2 * sizeof(double));
  if (!tmp) return fail(GATO_ENOMEM, "scratch");
  GATO_TRY(poisson_run(plan->p, a, EPI_ENERGY, false, tmp, as_stream(stream)));
  GATO_CUDA_TRY(cudaMemcpyAsync(E_dev, tmp, sizeof(double), cudaMemcpyDeviceToDevice,
                                as_stream(stream)));
  return GATO_OK;
}

namespace gato {
// Matvec exchange: out += coef * sum_j phi_j J[phi_j psi] (scf.py:66-85).
int exchange_args(PassArgs& a, const void* psi, const void* orbitals, int n_orb, size_t esz,
                  int64_t n3, void* out, double coef) {
  if (n_orb + 1 > kMaxIn) return fail(GATO_EUNSUPPORTED, "exchange: at most %d orbitals", kMaxIn - 1);
  for (int j = 0; j < n_orb; ++j) a.in[j] = (const char*)orbitals + (size_t)j * n3 * esz;
  a.in[n_orb] = psi;
  a.out[0] = out;
  a.nout = 1;
  a.nf = (n_orb + 1) / 2;
  for (int j = 0; j < n_orb; ++j) {
    PartDesc& d = a.f[j / 2].p[j % 2];
    d.a = (int8_t)j;
    d.b = (int8_t)n_orb;
    d.nt = 1;
    d.to[0] = 0;
    d.tc[0] = (int8_t)j;
    d.coef[0] = (float)coef;
  }
  return GATO_OK;
}
}  // namespace gato

extern "C" int gato_exchange_apply(gato_poisson_t plan, const void* psi, const void* orbitals,
                                   int n_orb, void* out, double coef, void* stream) {
  if (!plan || !psi || !orbitals || !out || n_orb < 1)
    return fail(GATO_EBADARG, "gato_exchange_apply: bad arguments");
  PassArgs a;
  const size_t esz = plan->p.dtype == GATO_F64 ? 8 : 4;
  const int64_t n3 = (int64_t)plan->p.N * plan->p.N * plan->p.N;
  GATO_TRY(exchange_args(a, psi, orbitals, n_orb, esz, n3, out, coef));
  return poisson_run(plan->p, a, EPI_ACC, true, nullptr, as_stream(stream));
}

// Profiling hook: one strided stage of the pipeline on the plan's own
// spectral buffers (whatever they hold), so a caller can time it alone.
extern "C" int gato_poisson_stage(gato_poisson_t plan, int stage, int nf, void* stream) {
  if (!plan || stage < 1 || stage > 3 || nf < 1 || nf > plan->p.max_fields)
    return fail(GATO_EBADARG, "gato_poisson_stage: bad arguments");
  PoissonPlan& pl = plan->p;
  const int N = pl.N, M = pl.M;
  const int64_t nrows = (int64_t)N * N;
  cudaStream_t s = as_stream(stream);
  auto run = [&](auto* S1, auto* S2, auto* tw, auto* tw2, auto* ghat) -> int {
    using T2 = std::remove_pointer_t<decltype(S1)>;
    using T = std::remove_const_t<std::remove_pointer_t<decltype(ghat)>>;
    const int mode = stage == 1 ? COL_FWD : (stage == 2 ? COL_FMI : COL_INV);
    if constexpr (sizeof(T) == 4) {
      if (pl.engine != 1 && pl.engine != 4 && pl.tw4 && fast::rows_L<T>(M) > 0) {
        ColGeom g1{nrows * M, (int64_t)N * M * M, (int64_t)N * M, (int64_t)M * M, M, M, M, N, M};
        ColGeom g2{(int64_t)N * M * M, (int64_t)N * M * M, M, M, (int64_t)M * M, (int64_t)M * M, M, N, N};
        ColGeom g3{(int64_t)N * M * M, nrows * M, (int64_t)M * M, (int64_t)N * M, M, M, M, M, N};
        return fast::packed_cols(M, mode, stage == 1 ? (const float2*)S1 : (const float2*)S2,
                                 stage == 3 ? (float2*)S1 : (float2*)S2, stage == 1 ? g1 : (stage == 2 ? g2 : g3),
                                 stage == 2 ? M : N, nf, (const float4*)pl.tw4,
                                 stage == 2 ? (const float*)pl.ghat2 : nullptr, pl.H, s);
      }
    }
    if (pl.engine != 1 && fast::rows_L<T>(M) > 0) {
      ColGeom g1{nrows * M, (int64_t)N * M * M, (int64_t)N * M, (int64_t)M * M, M, M, M, N, M};
      ColGeom g2{(int64_t)N * M * M, (int64_t)N * M * M, M, M, (int64_t)M * M, (int64_t)M * M, M, N, N};
      ColGeom g3{(int64_t)N * M * M, nrows * M, (int64_t)M * M, (int64_t)N * M, M, M, M, M, N};
      return fast::cols<T>(M, mode, stage == 1 ? S1 : S2, stage == 3 ? S1 : S2,
                           stage == 1 ? g1 : (stage == 2 ? g2 : g3), stage == 2 ? M : N, nf, tw2,
                           stage == 2 ? ghat : nullptr, pl.H, s);
    }
    if (stage == 1) {
      ColGeom g{nrows * M, (int64_t)N * M * M, (int64_t)N * M, (int64_t)M * M, M, M, M, N, M};
      return launch_cols<T2>(COL_FWD, S1, S2, g, N, nf, pl.fp, tw, nullptr, pl.H, s);
    }
    if (stage == 2) {
      ColGeom g{(int64_t)N * M * M, (int64_t)N * M * M, M, M, (int64_t)M * M, (int64_t)M * M, M, N, N};
      return launch_cols<T2>(COL_FMI, S2, S2, g, M, nf, pl.fp, tw, ghat, pl.H, s);
    }
    ColGeom g{(int64_t)N * M * M, nrows * M, (int64_t)M * M, (int64_t)N * M, M, M, M, M, N};
    return launch_cols<T2>(COL_INV, S2, S1, g, N, nf, pl.fp, tw, nullptr, pl.H, s);
  };
  if (pl.dtype == GATO_F64)
    return run((double2*)pl.S1, (double2*)pl.S2, (const double2*)pl.tw, (const double2*)pl.tw2,
               (const double*)pl.ghat);
  return run((float2*)pl.S1, (float2*)pl.S2, (const float2*)pl.tw, (const float2*)pl.tw2, (const float*)pl.ghat);
}

// Tuning knobs: fields per launch group (1..max_fields, 0 = all) and the FFT
// engine (0: register-resident two-pass kernels where M has one, with the
// multi-field z forward for groups of two or more fields; 1: generic; 2: the
// register kernels with one z-forward CTA per field; 3: the register kernels
// with the multi-field z forward from three fields; 4: as 0, with the scalar
// FP32 column passes instead of the packed two-line ones and the z forward
// staging once per CTA instead of persistent CTAs with double-buffered staging).
extern "C" int gato_poisson_tune(gato_poisson_t plan, int group, int engine) {
  if (!plan || group < 0 || group > plan->p.max_fields || engine < 0 || engine > 4)
    return fail(GATO_EBADARG, "gato_poisson_tune: bad arguments");
  plan->p.group = group;
  plan->p.engine = engine;
  return GATO_OK;
}

namespace gato {
bool poisson_j_supported(const PoissonPlan& pl) {
  if (pl.engine == 1) return false;
  return (pl.dtype == GATO_F64 ? fast::rows_L<double>(pl.M) : fast::rows_L<float>(pl.M)) > 0;
}

bool poisson_fe_supported(const PoissonPlan& pl) {
  return pl.dtype == GATO_F64 && poisson_j_supported(pl);
}

namespace {
// out_a -= sum over pairs (a, b) of phi_b J_ab (each J read once). V is the
// element group a thread moves per field: a 16-byte vector where every field
// starts on a 16-byte boundary and n3 divides into vectors, else one element.
template <typename T, int NORB, int V>
__global__ void k_pair_exchange(const T* __restrict__ orb, const T* __restrict__ J, T* out, int64_t n3) {
  using VT = typename std::conditional<V == 1, T,
             typename std::conditional<sizeof(T) == 4, float4, double2>::type>::type;
  const int64_t nv = n3 / V;
  const VT* o4 = reinterpret_cast<const VT*>(orb);
  const VT* j4 = reinterpret_cast<const VT*>(J);
  VT* r4 = reinterpret_cast<VT*>(out);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv;
       i += (int64_t)gridDim.x * blockDim.x) {
    VT phiv[NORB];
    T acc[NORB][V];
#pragma unroll
    for (int a = 0; a < NORB; ++a) {
      phiv[a] = o4[(int64_t)a * nv + i];
#pragma unroll
      for (int u = 0; u < V; ++u) acc[a][u] = (T)0;
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < NORB; ++a)
#pragma unroll
      for (int b = a; b < NORB; ++b, ++k) {
        const VT jv = j4[(int64_t)k * nv + i];
        const T* j = reinterpret_cast<const T*>(&jv);
        const T* pa = reinterpret_cast<const T*>(&phiv[a]);
        const T* pb = reinterpret_cast<const T*>(&phiv[b]);
#pragma unroll
        for (int u = 0; u < V; ++u) {
          acc[a][u] += pb[u] * j[u];
          if (b != a) acc[b][u] += pa[u] * j[u];
        }
      }
#pragma unroll
    for (int a = 0; a < NORB; ++a) {
      VT r = r4[(int64_t)a * nv + i];
      T* re = reinterpret_cast<T*>(&r);
#pragma unroll
      for (int u = 0; u < V; ++u) re[u] -= acc[a][u];
      r4[(int64_t)a * nv + i] = r;
    }
  }
}

template <typename T>
int pair_exchange_t(const T* orb, int n, const T* J, T* out, int64_t n3, cudaStream_t s) {
  constexpr int VEC = 16 / (int)sizeof(T);
  const bool vec = n3 % VEC == 0 && (uintptr_t)orb % 16 == 0 && (uintptr_t)J % 16 == 0 &&
                   (uintptr_t)out % 16 == 0;
  const unsigned g = grid_for(vec ? n3 / VEC : n3, 256, 152 * 8);
  switch (n) {
#define GATO_PX(NN)                                                          \
  case NN:                                                                   \
    if (vec) k_pair_exchange<T, NN, VEC><<<g, 256, 0, s>>>(orb, J, out, n3); \
    else k_pair_exchange<T, NN, 1><<<g, 256, 0, s>>>(orb, J, out, n3);       \
    break;
    GATO_PX(1) GATO_PX(2) GATO_PX(3) GATO_PX(4) GATO_PX(5) GATO_PX(6) GATO_PX(7) GATO_PX(8)
#undef GATO_PX
    default: return fail(GATO_EUNSUPPORTED, "pair exchange: at most 8 orbitals");
  }
  GATO_LAUNCH_TRY();
  return GATO_OK;
}
}  // namespace

int pair_exchange(int dtype, const void* orbitals, int n, const void* J, void* out, int64_t n3,
                  cudaStream_t s) {
  if (dtype == GATO_F64)
    return pair_exchange_t<double>((const double*)orbitals, n, (const double*)J, (double*)out, n3, s);
  return pair_exchange_t<float>((const float*)orbitals, n, (const float*)J, (float*)out, n3, s);
}
}  // namespace gato
