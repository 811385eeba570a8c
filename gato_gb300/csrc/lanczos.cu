// Lanczos with full reorthogonalisation (solvers/lanczos.py:110-206).
//
// The m-step loop runs on the device with no host synchronisation: every
// scalar (alpha_j, beta_j, Gram-Schmidt coefficients) lives in device memory
// and is read by the next kernel. Per step:
//   F v_j -> W (the operator writes straight into the Krylov slot j+1)
//   alpha  : alpha_j = dV <v_j, W - beta_{j-1} v_{j-1}>
//   gemv_t : c_k = dV <v_k, w''>, w'' = W - beta_{j-1} v_{j-1} - alpha_j v_j, k <= j
//   gemv_n : W <- w'' - sum_k c_k v_k, with |W|^2 partials
//   [further classical Gram-Schmidt passes when reorth_passes > 1]
//   scale  : beta_j = sqrt(dV |W|^2), v_{j+1} = W / beta_j (zero if beta_j = 0)
// This is the reference's three-term step followed by a Gram-Schmidt sweep
// against v_0..v_j; the classical sweep reads the basis twice per step in
// two launches where modified Gram-Schmidt needs one dependent pass per
// vector, and (with the three-term part removed first) it keeps the basis
// orthogonal to working precision.
//
// The m x m tridiagonal eigenproblem is solved on the device in FP64:
// eigenvalue k by multisection on the Sturm count (32 lanes bisect at once),
// eigenvectors by inverse iteration with the partial-pivoting tridiagonal LU
// (the LAPACK dgttrf/dgtts2 scheme), re-orthogonalised within clusters of
// close eigenvalues. Ritz vectors are sum_j Y[j,k] v_j.
#include <atomic>
#include <cmath>
#include <type_traits>

#include <cuda.h>

#include "op.cuh"
#include "ptx.cuh"

namespace gato {
int dot_impl(int dtype, const void* a, const void* b, int64_t n, double scale, double* out,
             cudaStream_t s);
}

namespace gato {

namespace {

constexpr int kLzThreads = 256;
constexpr int kEPT = 8;                         // elements per thread per chunk
constexpr int kChunk = kLzThreads * kEPT;       // elements per block-chunk

// Up to two vectors subtracted from W on the fly: w = W - s0 u0 - s1 u1, the
// scalars read from device memory (beta_{j-1} and alpha_j of the step).
template <typename T>
struct Pre {
  const T* u[2] = {nullptr, nullptr};
  const double* s[2] = {nullptr, nullptr};
};

template <typename T>
__device__ __forceinline__ void pre_scalars(const Pre<T>& p, T* sc) {
  sc[0] = p.u[0] ? (T)p.s[0][0] : (T)0;
  sc[1] = p.u[1] ? (T)p.s[1][0] : (T)0;
}

template <typename T>
__device__ __forceinline__ T pre_load(const T* W, const Pre<T>& p, const T* sc, int64_t i) {
  T w = W[i];
  if (p.u[0]) w -= sc[0] * p.u[0][i];
  if (p.u[1]) w -= sc[1] * p.u[1][i];
  return w;
}

// c_k partials: part[k * nblk + block] = sum_i V_k[i] w[i]. C is the type the
// per-vector products and warp sums run in; the launches use the field type:
// c_k is a cancellation sum (nearly orthogonal vectors), so its error scales
// with |w|, not with c_k, and FP32 products would leave 1e-9-level components
// in an FP64 basis.
// Each block owns one contiguous, equal share of the n elements (rounded to
// whole warps), walked in chunks of kChunk; basis vectors go four at a time
// so every thread has 4 * kEPT independent loads in flight per step.
__device__ __forceinline__ void block_range(int64_t n, int64_t& lo, int64_t& hi) {
  int64_t per = (n + gridDim.x - 1) / gridDim.x;
  per = (per + 31) / 32 * 32;
  lo = (int64_t)blockIdx.x * per;
  hi = lo + per < n ? lo + per : n;
}

template <typename C>
__device__ __forceinline__ double warp_total(C v) {
  if constexpr (sizeof(C) == 4) return (double)warp_sumf(v);
  else return warp_sum(v);
}

template <typename T, typename C>
__global__ void __launch_bounds__(kLzThreads)
    k_gemv_t(const T* __restrict__ V, int64_t ld, int nk, const T* __restrict__ W, Pre<T> pre,
             int64_t n, double* part) {
  extern __shared__ double wacc[];   // [warp][k]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kLzThreads / 32;
  T sc[2];
  pre_scalars(pre, sc);
  for (int i = threadIdx.x; i < nw * nk; i += blockDim.x) wacc[i] = 0.0;
  __syncthreads();
  int64_t lo, hi;
  block_range(n, lo, hi);
  for (int64_t base = lo; base < hi; base += kChunk) {
    C w[kEPT];
#pragma unroll
    for (int e = 0; e < kEPT; ++e) {
      const int64_t i = base + e * kLzThreads + threadIdx.x;
      w[e] = i < hi ? (C)pre_load(W, pre, sc, i) : (C)0;
    }
    int k = 0;
    for (; k + 4 <= nk; k += 4) {
      C sk[4] = {(C)0, (C)0, (C)0, (C)0};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const T* vk = V + (int64_t)(k + u) * ld;
#pragma unroll
        for (int e = 0; e < kEPT; ++e) {
          const int64_t i = base + e * kLzThreads + threadIdx.x;
          if (i < hi) sk[u] = fma((C)vk[i], w[e], sk[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double d = warp_total<C>(sk[u]);
        if (lane == 0) wacc[warp * nk + k + u] += d;
      }
    }
    for (; k < nk; ++k) {
      const T* vk = V + (int64_t)k * ld;
      C sk = (C)0;
#pragma unroll
      for (int e = 0; e < kEPT; ++e) {
        const int64_t i = base + e * kLzThreads + threadIdx.x;
        if (i < hi) sk = fma((C)vk[i], w[e], sk);
      }
      const double d = warp_total<C>(sk);
      if (lane == 0) wacc[warp * nk + k] += d;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += wacc[w * nk + k];
    part[(int64_t)k * gridDim.x + blockIdx.x] = s;
  }
}

// W <- W - pre - sum_k c_k v_k ; norm partials part[block]. The correction
// sum_k c_k v_k is formed in C and subtracted in T. Launched with C = float:
// once the three-term part is removed the c_k are roundoff-sized (about
// 1e-14 |w| in FP64), so rounding each term to FP32 perturbs w far below its
// own last digit, while GB300's narrow FP64 pipe would otherwise spend one
// DFMA per element per basis vector here.
template <typename T, typename C>
__global__ void __launch_bounds__(kLzThreads)
    k_gemv_n(const T* __restrict__ V, int64_t ld, int nk, T* __restrict__ W, Pre<T> pre,
             const double* __restrict__ c, int64_t n, double* part) {
  extern __shared__ double cs[];
  __shared__ double sh[32];
  for (int k = threadIdx.x; k < nk; k += blockDim.x) cs[k] = c[k];
  __syncthreads();
  T sc[2];
  pre_scalars(pre, sc);
  Acc<T> acc;
  int64_t lo, hi;
  block_range(n, lo, hi);
  for (int64_t base = lo; base < hi; base += kChunk) {
    T w[kEPT];
    C corr[kEPT];
#pragma unroll
    for (int e = 0; e < kEPT; ++e) {
      const int64_t i = base + e * kLzThreads + threadIdx.x;
      w[e] = i < hi ? pre_load(W, pre, sc, i) : (T)0;
      corr[e] = (C)0;
    }
    int k = 0;
    for (; k + 4 <= nk; k += 4) {
      C v[4][kEPT];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const T* vk = V + (int64_t)(k + u) * ld;
#pragma unroll
        for (int e = 0; e < kEPT; ++e) {
          const int64_t i = base + e * kLzThreads + threadIdx.x;
          v[u][e] = i < hi ? (C)vk[i] : (C)0;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const C ck = (C)cs[k + u];
#pragma unroll
        for (int e = 0; e < kEPT; ++e) corr[e] = fma(ck, v[u][e], corr[e]);
      }
    }
    for (; k < nk; ++k) {
      const T* vk = V + (int64_t)k * ld;
      const C ck = (C)cs[k];
#pragma unroll
      for (int e = 0; e < kEPT; ++e) {
        const int64_t i = base + e * kLzThreads + threadIdx.x;
        if (i < hi) corr[e] = fma(ck, (C)vk[i], corr[e]);
      }
    }
#pragma unroll
    for (int e = 0; e < kEPT; ++e) {
      const int64_t i = base + e * kLzThreads + threadIdx.x;
      if (i < hi) {
        w[e] -= (T)corr[e];
        W[i] = w[e];
        acc.add_prod(w[e], w[e]);
      }
    }
  }
  const double s = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// ---- bulk-copy streaming versions of the two sweeps ----------------------------
// The basis vectors are the bulk of the Lanczos traffic. Here each block owns
// an equal element range; a producer warp's lane 0 streams the items (chunk c,
// vector k) of that range, chunk-major, as contiguous 1-D bulk copies into a
// kBulkStages ring (one "full" mbarrier per stage with the byte count, one
// "empty" mbarrier with one arrival per consumer warp). The eight consumer
// warps read each item from shared memory as 16-byte vectors, release the stage
// at once, and do the arithmetic in registers: the memory parallelism lives
// in the ring (48 KB per block) instead of in registers. Used when every
// vector starts on a 16-byte boundary and n * sizeof(T) is a multiple of 16.
constexpr int kBulkStages = 6;   // 48 KB of ring per block: 3 blocks per SM
constexpr int kBulkWarps = 8;                           // consumer warps
constexpr int kBulkThreads = 32 * (kBulkWarps + 1);     // + the producer warp

template <typename T>
struct BulkGeom {
  static constexpr int VEC = 16 / (int)sizeof(T);          // elements per 16-byte vector
  static constexpr int CH = sizeof(T) == 4 ? 2048 : 1024;  // elements per item (8 KB)
  static constexpr int GRP = CH / (32 * kBulkWarps * VEC); // vectors per thread per item (2)
  static constexpr int EPT = GRP * VEC;
  // element u of group g of consumer thread ct sits at g * (256 VEC) + ct VEC + u
  __device__ static int idx(int ct, int g, int u) { return g * (32 * kBulkWarps * VEC) + ct * VEC + u; }
};

template <typename T>
__device__ __forceinline__ void bulk_producer(const T* V, int64_t ld, int nk, int64_t lo, int64_t hi,
                                              int items, T* stage, uint64_t* full, uint64_t* empty,
                                              volatile int* abort_v, int* err) {
  using G = BulkGeom<T>;
  int t = 0, c = 0, k = 0;
  for (; t < items; ++t) {
    const int sl = t % kBulkStages;
    if (t >= kBulkStages &&
        !mbar_wait_bounded(&empty[sl], (uint32_t)(((t / kBulkStages) - 1) & 1), err, 105)) {
      *abort_v = 1;
      break;
    }
    if (*abort_v) break;
    const int64_t base = lo + (int64_t)c * G::CH;
    const int64_t cnt = hi - base < G::CH ? hi - base : G::CH;
    const uint32_t bytes = (uint32_t)(cnt * sizeof(T));
    mbar_expect_tx(&full[sl], bytes);
    bulk_load(stage + (size_t)sl * G::CH, V + (int64_t)k * ld + base, bytes, &full[sl]);
    if (++k == nk) {
      k = 0;
      ++c;
    }
  }
  if (*abort_v)   // let the copies in flight land (bounded) before the block exits
    for (int p = t > kBulkStages ? t - kBulkStages : 0; p < t; ++p)
      mbar_wait_bounded(&full[p % kBulkStages], (uint32_t)((p / kBulkStages) & 1), err, 106);
}

// Warp-uniform wait for item t; false (and the abort flag set) if it timed out.
__device__ __forceinline__ bool bulk_wait(uint64_t* full, int t, volatile int* abort_v, int* err) {
  bool fail = *abort_v != 0;
  if (!fail) fail = !mbar_wait_bounded(&full[t % kBulkStages], (uint32_t)((t / kBulkStages) & 1), err, 107);
  if (__any_sync(0xffffffffu, fail)) {
    if ((threadIdx.x & 31) == 0) *abort_v = 1;
    return false;
  }
  return true;
}

// k_gemv_t with bulk streaming: part[k * gridDim.x + block] = sum_i V_k[i] w[i]
template <typename T>
__global__ void __launch_bounds__(kBulkThreads)
    k_gemv_t_bulk(const T* __restrict__ V, int64_t ld, int nk, const T* __restrict__ W, Pre<T> pre,
                  int64_t n, double* part, int* err) {
  using G = BulkGeom<T>;
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  extern __shared__ __align__(128) unsigned char smb[];
  T* stage = reinterpret_cast<T*>(smb);
  uint64_t* full = reinterpret_cast<uint64_t*>(smb + (size_t)kBulkStages * G::CH * sizeof(T));
  uint64_t* empty = full + kBulkStages;
  double* wacc = reinterpret_cast<double*>(empty + kBulkStages);   // [warp][k]
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t lo, hi;
  block_range(n, lo, hi);
  const int nch = hi > lo ? (int)((hi - lo + G::CH - 1) / G::CH) : 0;
  const int items = nch * nk;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kBulkStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kBulkWarps);
    }
    abort_flag = 0;
    fence_barrier_init();
  }
  for (int i = threadIdx.x; i < kBulkWarps * nk; i += blockDim.x) wacc[i] = 0.0;
  __syncthreads();
  if (warp == kBulkWarps) {
    if (lane == 0) bulk_producer<T>(V, ld, nk, lo, hi, items, stage, full, empty, abort_v, err);
  } else {
    const int ct = threadIdx.x;
    T sc[2];
    pre_scalars(pre, sc);
    T w[G::EPT];
    int c = 0, k = 0;
    for (int t = 0; t < items; ++t) {
      const int64_t base = lo + (int64_t)c * G::CH;
      if (k == 0) {
#pragma unroll
        for (int g = 0; g < G::GRP; ++g)
#pragma unroll
          for (int u = 0; u < G::VEC; ++u) {
            const int64_t i = base + G::idx(ct, g, u);
            w[g * G::VEC + u] = i < hi ? pre_load(W, pre, sc, i) : (T)0;
          }
      }
      if (!bulk_wait(full, t, abort_v, err)) break;
      const T* st = stage + (size_t)(t % kBulkStages) * G::CH;
      T v[G::EPT];
#pragma unroll
      for (int g = 0; g < G::GRP; ++g) {
        const V4 q = *reinterpret_cast<const V4*>(st + G::idx(ct, g, 0));
        const T* qe = reinterpret_cast<const T*>(&q);
#pragma unroll
        for (int u = 0; u < G::VEC; ++u) v[g * G::VEC + u] = qe[u];
      }
      fence_proxy_async_smem();   // the slot's reads are done before the next bulk copy lands
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[t % kBulkStages]);
      T sk = (T)0;
#pragma unroll
      for (int g = 0; g < G::GRP; ++g)
#pragma unroll
        for (int u = 0; u < G::VEC; ++u)
          if (base + G::idx(ct, g, u) < hi) sk = fma(v[g * G::VEC + u], w[g * G::VEC + u], sk);
      const double d = warp_total<T>(sk);
      if (lane == 0) wacc[warp * nk + k] += d;
      if (++k == nk) {
        k = 0;
        ++c;
      }
    }
  }
  __syncthreads();
  if (*abort_v) return;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    double sum = 0.0;
    for (int wp = 0; wp < kBulkWarps; ++wp) sum += wacc[wp * nk + k];
    part[(int64_t)k * gridDim.x + blockIdx.x] = sum;
  }
}

// Vector-major variant of k_gemv_t_bulk for blocks whose range spans at most
// kVmChunks chunks: the producer streams item t = k * nch + c (all chunks of
// vector k, then vector k + 1), each consumer thread keeps w for every chunk
// of the range in registers, accumulates vector k over its chunks and reduces
// it across the warp once, with a plain store of the warp's partial. The
// chunk-major kernel instead reduces every item and adds it to shared memory
// in FP64, a dependent FP64 step per item on GB300's narrow FP64 pipe.
constexpr int kVmChunks = 4;

template <typename T>
__device__ __forceinline__ void bulk_producer_vm(const T* V, int64_t ld, int nk, int64_t lo, int64_t hi,
                                                 int nch, T* stage, uint64_t* full, uint64_t* empty,
                                                 volatile int* abort_v, int* err) {
  using G = BulkGeom<T>;
  const int items = nk * nch;
  int t = 0;
  for (int k = 0; k < nk && !*abort_v; ++k)
    for (int c = 0; c < nch; ++c, ++t) {
      const int sl = t % kBulkStages;
      if (t >= kBulkStages &&
          !mbar_wait_bounded(&empty[sl], (uint32_t)(((t / kBulkStages) - 1) & 1), err, 105)) {
        *abort_v = 1;
        break;
      }
      if (*abort_v) break;
      const int64_t base = lo + (int64_t)c * G::CH;
      const int64_t cnt = hi - base < G::CH ? hi - base : G::CH;
      const uint32_t bytes = (uint32_t)(cnt * sizeof(T));
      mbar_expect_tx(&full[sl], bytes);
      bulk_load(stage + (size_t)sl * G::CH, V + (int64_t)k * ld + base, bytes, &full[sl]);
    }
  (void)items;
  if (*abort_v)   // let the copies in flight land (bounded) before the block exits
    for (int p = t > kBulkStages ? t - kBulkStages : 0; p < t; ++p)
      mbar_wait_bounded(&full[p % kBulkStages], (uint32_t)((p / kBulkStages) & 1), err, 106);
}

template <typename T>
__global__ void __launch_bounds__(kBulkThreads, 3)
    k_gemv_t_vm(const T* __restrict__ V, int64_t ld, int nk, const T* __restrict__ W, Pre<T> pre,
                int64_t n, double* part, int* err) {
  using G = BulkGeom<T>;
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  extern __shared__ __align__(128) unsigned char smb[];
  T* stage = reinterpret_cast<T*>(smb);
  uint64_t* full = reinterpret_cast<uint64_t*>(smb + (size_t)kBulkStages * G::CH * sizeof(T));
  uint64_t* empty = full + kBulkStages;
  double* wacc = reinterpret_cast<double*>(empty + kBulkStages);   // [warp][k]
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t lo, hi;
  block_range(n, lo, hi);
  const int nch = hi > lo ? (int)((hi - lo + G::CH - 1) / G::CH) : 0;   // <= kVmChunks (host-checked)
  if (threadIdx.x == 0) {
    for (int i = 0; i < kBulkStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kBulkWarps);
    }
    abort_flag = 0;
    fence_barrier_init();
  }
  for (int i = threadIdx.x; i < kBulkWarps * nk; i += blockDim.x) wacc[i] = 0.0;
  __syncthreads();
  if (warp == kBulkWarps) {
    if (lane == 0) bulk_producer_vm<T>(V, ld, nk, lo, hi, nch, stage, full, empty, abort_v, err);
  } else {
    const int ct = threadIdx.x;
    T sc[2];
    pre_scalars(pre, sc);
    // w for every chunk of the range; elements past hi are zero
    T w[kVmChunks][G::EPT];
    int lim[kVmChunks];   // valid elements of chunk c
#pragma unroll
    for (int c = 0; c < kVmChunks; ++c) {
      const int64_t base = lo + (int64_t)c * G::CH;
      lim[c] = c < nch ? (int)(hi - base < G::CH ? hi - base : G::CH) : 0;
#pragma unroll
      for (int g = 0; g < G::GRP; ++g)
#pragma unroll
        for (int u = 0; u < G::VEC; ++u) {
          const int li = G::idx(ct, g, u);
          w[c][g * G::VEC + u] = li < lim[c] ? pre_load(W, pre, sc, base + li) : (T)0;
        }
    }
    int t = 0;
    bool ok = true;
    for (int k = 0; k < nk && ok; ++k) {
      T sk = (T)0;
#pragma unroll
      for (int c = 0; c < kVmChunks; ++c) {
        if (c >= nch) break;
        if (!bulk_wait(full, t, abort_v, err)) {
          ok = false;
          break;
        }
        const T* st = stage + (size_t)(t % kBulkStages) * G::CH;
        T v[G::EPT];
#pragma unroll
        for (int g = 0; g < G::GRP; ++g) {
          const V4 q = *reinterpret_cast<const V4*>(st + G::idx(ct, g, 0));
          const T* qe = reinterpret_cast<const T*>(&q);
#pragma unroll
          for (int u = 0; u < G::VEC; ++u) v[g * G::VEC + u] = qe[u];
        }
        fence_proxy_async_smem();   // the slot's reads are done before the next bulk copy lands
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[t % kBulkStages]);
        ++t;
        const bool whole = lim[c] == G::CH;
#pragma unroll
        for (int g = 0; g < G::GRP; ++g)
#pragma unroll
          for (int u = 0; u < G::VEC; ++u)
            if (whole || G::idx(ct, g, u) < lim[c]) sk = fma(v[g * G::VEC + u], w[c][g * G::VEC + u], sk);
      }
      if (!ok) break;
      const double d = warp_total<T>(sk);
      if (lane == 0) wacc[warp * nk + k] = d;
    }
  }
  __syncthreads();
  if (*abort_v) return;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    double sum = 0.0;
    for (int wp = 0; wp < kBulkWarps; ++wp) sum += wacc[wp * nk + k];
    part[(int64_t)k * gridDim.x + blockIdx.x] = sum;
  }
}

// k_gemv_n with bulk streaming: W <- W - pre - sum_k c_k v_k, norm partial
// part[block]; the correction accumulates in FP32 as in k_gemv_n<T, float>.
template <typename T>
__global__ void __launch_bounds__(kBulkThreads)
    k_gemv_n_bulk(const T* __restrict__ V, int64_t ld, int nk, T* __restrict__ W, Pre<T> pre,
                  const double* __restrict__ c_in, int64_t n, double* part, int* err) {
  using G = BulkGeom<T>;
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  extern __shared__ __align__(128) unsigned char smb[];
  T* stage = reinterpret_cast<T*>(smb);
  uint64_t* full = reinterpret_cast<uint64_t*>(smb + (size_t)kBulkStages * G::CH * sizeof(T));
  uint64_t* empty = full + kBulkStages;
  float* cs = reinterpret_cast<float*>(empty + kBulkStages);   // coefficients rounded once to FP32
  __shared__ double sh[32];
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t lo, hi;
  block_range(n, lo, hi);
  const int nch = hi > lo ? (int)((hi - lo + G::CH - 1) / G::CH) : 0;
  const int items = nch * nk;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kBulkStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kBulkWarps);
    }
    abort_flag = 0;
    fence_barrier_init();
  }
  for (int i = threadIdx.x; i < nk; i += blockDim.x) cs[i] = (float)c_in[i];
  __syncthreads();
  Acc<T> acc;
  if (warp == kBulkWarps) {
    if (lane == 0) bulk_producer<T>(V, ld, nk, lo, hi, items, stage, full, empty, abort_v, err);
  } else {
    const int ct = threadIdx.x;
    T sc[2];
    pre_scalars(pre, sc);
    T w[G::EPT];
    float corr[G::EPT];
    int c = 0, k = 0;
    for (int t = 0; t < items; ++t) {
      const int64_t base = lo + (int64_t)c * G::CH;
      if (k == 0) {
#pragma unroll
        for (int g = 0; g < G::GRP; ++g)
#pragma unroll
          for (int u = 0; u < G::VEC; ++u) {
            const int64_t i = base + G::idx(ct, g, u);
            w[g * G::VEC + u] = i < hi ? pre_load(W, pre, sc, i) : (T)0;
            corr[g * G::VEC + u] = 0.f;
          }
      }
      if (!bulk_wait(full, t, abort_v, err)) break;
      const T* st = stage + (size_t)(t % kBulkStages) * G::CH;
      T v[G::EPT];
#pragma unroll
      for (int g = 0; g < G::GRP; ++g) {
        const V4 q = *reinterpret_cast<const V4*>(st + G::idx(ct, g, 0));
        const T* qe = reinterpret_cast<const T*>(&q);
#pragma unroll
        for (int u = 0; u < G::VEC; ++u) v[g * G::VEC + u] = qe[u];
      }
      fence_proxy_async_smem();   // the slot's reads are done before the next bulk copy lands
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[t % kBulkStages]);
      const float ck = cs[k];
#pragma unroll
      for (int e = 0; e < G::EPT; ++e) corr[e] = fmaf(ck, (float)v[e], corr[e]);
      if (k == nk - 1) {
#pragma unroll
        for (int g = 0; g < G::GRP; ++g)
#pragma unroll
          for (int u = 0; u < G::VEC; ++u) {
            const int64_t i = base + G::idx(ct, g, u);
            if (i < hi) {
              const T x = w[g * G::VEC + u] - (T)corr[g * G::VEC + u];
              W[i] = x;
              acc.add_prod(x, x);
            }
          }
      }
      if (++k == nk) {
        k = 0;
        ++c;
      }
    }
  }
  const double sum = block_sum(acc.value(), sh);
  if (threadIdx.x == 0 && !*abort_v) part[blockIdx.x] = sum;
}

// nrm = dV * sum of the norm partials (the k_finalize_sums reduction order),
// beta = sqrt(nrm) -> binv[0] and betas_out[0], 1 / beta (0 if beta = 0) ->
// binv[1]: the FP64 square root and reciprocal once per step, in one thread.
__global__ void k_beta_finalize(const double* partials, int nparts, double scale, double* binv,
                                double* beta_out) {
  __shared__ double sh[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += partials[i];
  v = block_sum(v, sh);
  if (threadIdx.x == 0) {
    const double beta = sqrt(v * scale);
    binv[0] = beta;
    binv[1] = beta > 0 ? 1.0 / beta : 0.0;
    beta_out[0] = beta;
  }
}

// v = W / beta (or 0). The products run in the field type: an FP32 basis takes
// the FP64 reciprocal rounded once to FP32, as FP64 products would put three
// FP64-pipe operations on every element on GB300.
template <typename T>
__global__ void k_beta_scale(T* W, int64_t n, const double* binv) {
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  constexpr int VEC = 16 / (int)sizeof(T);
  const bool pos = binv[0] > 0;
  const T inv = (T)binv[1];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nv = ((uintptr_t)W % 16) == 0 ? n / VEC : 0;   // 16-byte vectors
  V* W4 = reinterpret_cast<V*>(W);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
    V v = W4[i];
    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
    for (int u = 0; u < VEC; ++u) e[u] = pos ? e[u] * inv : (T)0;
    W4[i] = v;
  }
  for (int64_t i = nv * VEC + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    W[i] = pos ? W[i] * inv : (T)0;
}

template <typename T>
__global__ void k_scale_copy(const T* __restrict__ src, T* dst, int64_t n, const double* nrm) {
  __shared__ double sc;   // one FP64 reciprocal square root per block
  if (threadIdx.x == 0) sc = 1.0 / sqrt(nrm[0]);
  __syncthreads();
  const T inv = (T)sc;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] * inv;
}


// ---- tridiagonal eigensolver (FP64) ----------------------------------------------

// Number of eigenvalues of T below x: the sign changes of the leading principal
// minors p_i = det(T_i - x I), p_0 = 1, p_1 = a_0 - x,
// p_{i+1} = (a_i - x) p_i - e_{i-1}^2 p_{i-1} (the Sturm sequence of Wilkinson,
// The Algebraic Eigenvalue Problem, ch. 5). No division: three FP64 operations
// a step instead of a division chain, which GB300's narrow FP64 pipe makes
// long. A zero minor takes the sign opposite to its predecessor (the LDL^T
// form's q_i = 0 -> -pivmin convention), and the pair (p_i, p_{i-1}) is
// rescaled by an exact power of two whenever p_i's exponent leaves [-480, 480].
__device__ int sturm_count(const double* a, const double* e2, int m, double x) {
  auto neg = [](double v, bool prev_neg) {
    const int hi = __double2hiint(v);
    const bool zero = ((hi & 0x7fffffff) | __double2loint(v)) == 0;
    return zero ? !prev_neg : hi < 0;
  };
  double pm = 1.0, p = a[0] - x;
  bool s = neg(p, false);
  int cnt = s;
  for (int i = 1; i < m; ++i) {
    const double pn = fma(a[i] - x, p, -e2[i - 1] * pm);
    const bool sn = neg(pn, s);
    cnt += sn != s;
    pm = p;
    p = pn;
    s = sn;
    const int ex = (__double2hiint(p) >> 20) & 0x7ff;
    if (ex > 1023 + 480) {
      p *= 0x1p-480;
      pm *= 0x1p-480;
    } else if (ex < 1023 - 480 && p != 0.0) {
      p *= 0x1p480;
      pm *= 0x1p480;
    }
  }
  return cnt;
}

// Gershgorin bound of T = diag(a) + offdiag(e): lower and upper ends and the
// norm max_i |a_i| + r_i (min/max are exact, so any reduction order agrees).
__device__ __forceinline__ void gershgorin(const double* a, const double* e, int m, double& lo, double& hi,
                                           double& nm) {
  lo = 1e300;
  hi = -1e300;
  nm = 0;
  for (int i = threadIdx.x; i < m; i += 32) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < m - 1 ? fabs(e[i]) : 0.0);
    lo = fmin(lo, a[i] - r);
    hi = fmax(hi, a[i] + r);
    nm = fmax(nm, fabs(a[i]) + r);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    nm = fmax(nm, __shfl_xor_sync(0xffffffffu, nm, o));
  }
}

// One warp per block, block k = eigenvalue k of T = diag(alpha) +
// offdiag(beta[:m-1]) (ascending). Multisection on Sturm counts (33
// sub-intervals a round), then inverse iteration: T - lambda_k I is factored
// once with partial pivoting (the LAPACK dgttrf scheme: multipliers,
// interchanges and reciprocal pivots kept in work) and the factors are applied
// to the iterate four times (dgtts2). One eigenvalue per block spreads the FP64
// work over K SMs: GB300's FP64 pipe is narrow, and a Sturm count is a chain
// of m dependent FP64 divisions. The factorisation and the iterate live in shared memory (each
// step of these sequential loops reads what the previous one wrote: in global memory every step
// would wait on a round trip through L2); the final vector goes to work + k*7m + 6m. Dynamic
// shared memory: a, e, e2 and d, du, du2, f, sw, rd, x, 10 m doubles.
__global__ void __launch_bounds__(32) k_tridiag_eig(const double* alpha, const double* beta, int m, int K,
                                                     double* lam_out, double* work, int* err) {
  extern __shared__ double sm[];
  double* a = sm;
  double* e = a + m;
  double* e2 = e + m;
  const int lane = threadIdx.x, k = blockIdx.x;
  for (int i = lane; i < m; i += 32) {
    a[i] = alpha[i];
    e[i] = i < m - 1 ? beta[i] : 0.0;
    e2[i] = e[i] * e[i];
  }
  __syncwarp();
  double glo, ghi, nm;
  gershgorin(a, e, m, glo, ghi, nm);
  const double pad = 2.2e-16 * nm * 4 + 1e-300;
  glo -= pad;
  ghi += pad;
  const double tnorm = nm > 0 ? nm : 1.0;
  const double pivmin = 1e-290 > 2.2e-16 * 2.2e-16 * tnorm ? 1e-290 : 1e-300;
  double lo = glo, hi = ghi;
  for (int it = 0; it < 80; ++it) {
    const double width = hi - lo;
    if (width <= 2.2e-16 * 2 * fmax(fabs(lo), fabs(hi)) + pivmin) break;
    const double x = lo + width * (double)(lane + 1) / 33.0;
    const int c = sturm_count(a, e2, m, x);
    // bracket: eigenvalue k lies in [x_i, x_{i+1}) where count(x_i) <= k < count(x_{i+1})
    const unsigned below = __ballot_sync(0xffffffffu, c <= k);   // lanes whose x is <= lambda_k
    const int nb = __popc(below);  // counts are monotone: lanes 0..nb-1 have c <= k
    const double nlo = nb > 0 ? lo + width * (double)nb / 33.0 : lo;
    const double nhi = nb < 32 ? lo + width * (double)(nb + 1) / 33.0 : hi;
    lo = nlo;
    hi = nhi;
  }
  if (lane != 0) return;
  const double shift = 0.5 * (lo + hi);
  lam_out[k] = shift;
  double* d = e2 + m;
  double* du = d + m;
  double* du2 = du + m;
  double* f = du2 + m;     // multiplier of step i
  double* sw = f + m;      // 1.0 where step i interchanged rows i and i+1
  double* rd = sw + m;     // 1 / d[i] of the final factor
  double* x = rd + m;
  const double tiny = 2.2e-16 * tnorm;
  for (int i = 0; i < m; ++i) {
    d[i] = a[i] - shift;
    du[i] = e[i];
    du2[i] = 0.0;
  }
  for (int i = 0; i < m - 1; ++i) {   // factor (dgttrf)
    const double dli = e[i];
    if (fabs(d[i]) >= fabs(dli)) {
      if (d[i] == 0.0) d[i] = tiny;
      f[i] = dli / d[i];
      sw[i] = 0.0;
      d[i + 1] -= f[i] * du[i];
      du2[i] = 0.0;
    } else {
      f[i] = d[i] / dli;
      sw[i] = 1.0;
      d[i] = dli;
      const double t = du[i];
      du[i] = d[i + 1];
      d[i + 1] = t - f[i] * d[i + 1];
      if (i < m - 2) {
        du2[i] = du[i + 1];
        du[i + 1] = -f[i] * du[i + 1];
      }
    }
  }
  if (d[m - 1] == 0.0) d[m - 1] = tiny;
  for (int i = 0; i < m; ++i) rd[i] = 1.0 / d[i];
  for (int i = 0; i < m; ++i) x[i] = 1.0 + 0.25 * sin(0.7 * (i + 1) * (k + 1) + 0.3);   // start vector
  for (int iter = 0; iter < 4; ++iter) {
    for (int i = 0; i < m - 1; ++i) {   // forward: L^-1 P x
      if (sw[i] == 0.0) {
        x[i + 1] -= f[i] * x[i];
      } else {
        const double xt = x[i];
        x[i] = x[i + 1];
        x[i + 1] = xt - f[i] * x[i + 1];
      }
    }
    x[m - 1] *= rd[m - 1];   // back substitution with U (diagonal, du, du2)
    if (m > 1) x[m - 2] = (x[m - 2] - du[m - 2] * x[m - 1]) * rd[m - 2];
    for (int i = m - 3; i >= 0; --i) x[i] = (x[i] - du[i] * x[i + 1] - du2[i] * x[i + 2]) * rd[i];
    double nrm = 0.0;
    for (int i = 0; i < m; ++i) nrm += x[i] * x[i];
    nrm = sqrt(nrm);
    if (!(nrm > 0) || !isfinite(nrm)) {
      if (err) atomicExch(err, 201);
      nrm = 1.0;
    }
    const double inv = 1.0 / nrm;
    for (int i = 0; i < m; ++i) x[i] *= inv;
  }
  double* xo = work + (int64_t)k * 7 * m + 6 * m;   // read by k_tridiag_finish
  for (int i = 0; i < m; ++i) xo[i] = x[i];
}

// Convergence flag (any beta_j < tol for j < max(m-1, 1), lanczos.py:199),
// re-orthogonalisation of eigenvectors of clustered eigenvalues, and the sign
// convention (largest component positive); writes evals and Y (column k at
// Y + k*m). One thread: O(K^2 m) work at most.
__global__ void k_tridiag_finish(const double* alpha, const double* beta, int m, int K, const double* lam,
                                 double* work, double* evals, double* Y, int* flag, double tol) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int fl = 0;
  const int lim = m - 1 > 1 ? m - 1 : 1;
  for (int j = 0; j < lim; ++j) fl |= beta[j] < tol;
  flag[0] = fl;
  double nm = 0;
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? fabs(beta[i - 1]) : 0.0) + (i < m - 1 ? fabs(beta[i]) : 0.0);
    nm = fmax(nm, fabs(alpha[i]) + r);
  }
  const double close = 1e-7 * (nm > 0 ? nm : 1.0);
  for (int k = 0; k < K; ++k) {
    double* xk = work + (int64_t)k * 7 * m + 6 * m;
    for (int l = 0; l < k; ++l) {
      if (fabs(lam[k] - lam[l]) > close) continue;
      const double* xl = work + (int64_t)l * 7 * m + 6 * m;
      double dot = 0;
      for (int i = 0; i < m; ++i) dot += xl[i] * xk[i];
      for (int i = 0; i < m; ++i) xk[i] -= dot * xl[i];
      double nrm = 0;
      for (int i = 0; i < m; ++i) nrm += xk[i] * xk[i];
      nrm = sqrt(nrm);
      for (int i = 0; i < m; ++i) xk[i] /= nrm;
    }
    int imax = 0;
    for (int i = 1; i < m; ++i)
      if (fabs(xk[i]) > fabs(xk[imax])) imax = i;
    const double sg = xk[imax] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < m; ++i) Y[(int64_t)k * m + i] = sg * xk[i];
    evals[k] = lam[k];
  }
}

// out[k] = sum_j Y[k*m + j] v_j for k in [k0, k0 + KB)
// The coefficients are rounded to the field type once, in shared memory (a
// conversion per product would run on GB300's narrow FP64 pipe), and eight
// basis loads per thread are in flight at a time.
template <typename T, int KB>
__global__ void __launch_bounds__(256) k_ritz(const T* __restrict__ V, int64_t ld, int m,
                                              const double* __restrict__ Y, int k0, int K,
                                              T* __restrict__ out, int64_t n) {
  extern __shared__ __align__(16) unsigned char ritz_sm[];
  T* ys = reinterpret_cast<T*>(ritz_sm);   // [KB][m]
  const int kb = min(KB, K - k0);
  for (int i = threadIdx.x; i < kb * m; i += blockDim.x) ys[i] = (T)Y[(int64_t)(k0 + i / m) * m + i % m];
  __syncthreads();
  constexpr int U = 8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    T acc[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) acc[k] = (T)0;
    int j = 0;
    for (; j + U <= m; j += U) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = V[(int64_t)(j + u) * ld + i];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int k = 0; k < KB; ++k)
          if (k < kb) acc[k] = fma(ys[k * m + j + u], v[u], acc[k]);
    }
    for (; j < m; ++j) {
      const T v = V[(int64_t)j * ld + i];
#pragma unroll
      for (int k = 0; k < KB; ++k)
        if (k < kb) acc[k] = fma(ys[k * m + j], v, acc[k]);
    }
#pragma unroll
    for (int k = 0; k < KB; ++k)
      if (k < kb) out[(int64_t)(k0 + k) * n + i] = acc[k];
  }
}

struct LzScratch {
  double *part, *coef, *nrm, *Y, *work;
  int nblk;     // k_gemv_n grid
  int nblk_t;   // k_gemv_t grid
  int nblk_b;   // bulk-streaming grid (both sweeps)
};

// One resident wave each: k_gemv_n holds 3 blocks of kLzThreads per SM (80
// registers); k_gemv_t, which is bound by memory latency, runs as many as its
// registers allow (48 FP32 / 62 FP64: 5 / 4 blocks) to keep more loads in flight.
inline int lz_nblk(int64_t n) { return (int)std::min<int64_t>((n + kChunk - 1) / kChunk, 3 * 152); }
inline int lz_nblk_t(int64_t n, bool fp64) {
  return (int)std::min<int64_t>((n + kChunk - 1) / kChunk, (fp64 ? 4 : 5) * 152);
}
// bulk-streaming kernels: 3 blocks per SM (their ring is 48 KB), at least one item each
inline int lz_nblk_b(int64_t n, bool fp64) {
  const int64_t ch = fp64 ? BulkGeom<double>::CH : BulkGeom<float>::CH;
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + ch - 1) / ch, 3 * 152));
}

int lz_scratch(cudaStream_t s, int64_t n, int m, int K, LzScratch& z, bool fp64) {
  z.nblk = lz_nblk(n);
  z.nblk_t = lz_nblk_t(n, fp64);
  z.nblk_b = lz_nblk_b(n, fp64);
  const int np = std::max(std::max(z.nblk, z.nblk_t), z.nblk_b);
  // partials (m+1)*max(grids), coefficients (m+1), norm, Y (m*K), LU work 7*m*K
  const size_t need = ((size_t)(m + 1) * np + (m + 1) + 8 + (size_t)m * K + (size_t)7 * m * K) *
                      sizeof(double);
  z.part = (double*)stream_scratch(s, need, kSlotLanczos);
  if (!z.part) return fail(GATO_ENOMEM, "lanczos: scratch allocation failed");
  z.coef = z.part + (size_t)(m + 1) * np;
  z.nrm = z.coef + (m + 1);
  z.Y = z.nrm + 8;
  z.work = z.Y + (size_t)m * K;
  return GATO_OK;
}

// v0 = psi0 / sqrt(<psi0, psi0> dV)
template <typename T>
int lz_begin(const void* psi0, T* Vb, int64_t n, double dV, const LzScratch& z, cudaStream_t s) {
  GATO_TRY(dot_impl(sizeof(T) == 8 ? GATO_F64 : GATO_F32, psi0, psi0, n, dV, z.nrm, s));
  k_scale_copy<T><<<grid_for(n, 256), 256, 0, s>>>((const T*)psi0, Vb, n, z.nrm);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

// Slot j+1 holds F v_j on entry and v_{j+1} on exit. The three-term part
// comes first, as in the reference: w' = F v_j - beta_{j-1} v_{j-1},
// alpha_j = <v_j, w'>, w'' = w' - alpha_j v_j; then classical Gram-Schmidt
// of w'' against v_0..v_j (reorth_passes times). Removing the large alpha_j
// component before the projection keeps one classical pass as orthogonal as
// the reference's modified Gram-Schmidt.
// The bulk kernels need every basis vector on a 16-byte boundary.
template <typename T>
bool bulk_ok(const T* Vb, int64_t n) {
  return ((uint64_t)n * sizeof(T)) % 16 == 0 && ((uintptr_t)Vb % 16) == 0;
}

// Opt in to the carve-out once per device and kernel (the kernels take up to
// ~64 KB). The flag is a static of this template's instantiation for the
// kernel itself: kernels of one signature must not share it.
template <auto Kern>
int bulk_smem_attr() {
  static std::atomic<unsigned> done{0};
  int dev = 0;
  GATO_CUDA_TRY(cudaGetDevice(&dev));
  const unsigned bit = 1u << (dev & 31);
  if (!(done.load() & bit)) {
    GATO_CUDA_TRY(cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
    done.fetch_or(bit);
  }
  return GATO_OK;
}

template <typename T>
int gemv_t_bulk(const T* V, int64_t ld, int nk, const T* W, const Pre<T>& pre, int64_t n, int nblk, double* part,
                cudaStream_t s) {
  const size_t sm = (size_t)kBulkStages * BulkGeom<T>::CH * sizeof(T) + 2 * kBulkStages * sizeof(uint64_t) +
                    (size_t)kBulkWarps * nk * sizeof(double);
  if (sm > 100 * 1024) return fail(GATO_EUNSUPPORTED, "lanczos: Krylov dimension too large for the bulk sweep");
  // the block range of block_range(): chunks per block decide the variant
  int64_t per = (n + nblk - 1) / nblk;
  per = (per + 31) / 32 * 32;
  if ((per + BulkGeom<T>::CH - 1) / BulkGeom<T>::CH <= kVmChunks) {
    GATO_TRY(bulk_smem_attr<k_gemv_t_vm<T>>());
    k_gemv_t_vm<T><<<nblk, kBulkThreads, sm, s>>>(V, ld, nk, W, pre, n, part, device_error_word());
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  GATO_TRY(bulk_smem_attr<k_gemv_t_bulk<T>>());
  k_gemv_t_bulk<T><<<nblk, kBulkThreads, sm, s>>>(V, ld, nk, W, pre, n, part, device_error_word());
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

template <typename T>
int gemv_n_bulk(const T* V, int64_t ld, int nk, T* W, const Pre<T>& pre, const double* c, int64_t n, int nblk,
                double* part, cudaStream_t s) {
  const size_t sm = (size_t)kBulkStages * BulkGeom<T>::CH * sizeof(T) + 2 * kBulkStages * sizeof(uint64_t) +
                    (size_t)nk * sizeof(double);
  GATO_TRY(bulk_smem_attr<k_gemv_n_bulk<T>>());
  k_gemv_n_bulk<T><<<nblk, kBulkThreads, sm, s>>>(V, ld, nk, W, pre, c, n, part, device_error_word());
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

template <typename T>
int lz_step(T* Vb, int64_t n, double dV, int j, int passes, double* alphas, double* betas,
            const LzScratch& z, cudaStream_t s) {
  T* W = Vb + (int64_t)(j + 1) * n;
  T* vj = Vb + (int64_t)j * n;
  Pre<T> p1;
  if (j > 0) {
    p1.u[0] = Vb + (int64_t)(j - 1) * n;
    p1.s[0] = betas + (j - 1);
  }
  const int nk = j + 1;
  if (bulk_ok(Vb, n)) {
    // alpha_j = dV <v_j, w'>
    GATO_TRY(gemv_t_bulk<T>(vj, n, 1, W, p1, n, z.nblk_b, z.part, s));
    GATO_TRY(finalize_sums(z.part, 1, z.nblk_b, dV, alphas + j, s));
    Pre<T> p2 = p1;
    p2.u[1] = vj;
    p2.s[1] = alphas + j;
    for (int p = 0; p < passes; ++p) {
      const Pre<T>& pp = p == 0 ? p2 : Pre<T>();
      GATO_TRY(gemv_t_bulk<T>(Vb, n, nk, W, pp, n, z.nblk_b, z.part, s));
      GATO_TRY(finalize_sums(z.part, nk, z.nblk_b, dV, z.coef, s));
      GATO_TRY(gemv_n_bulk<T>(Vb, n, nk, W, pp, z.coef, n, z.nblk_b, z.part, s));
    }
    k_beta_finalize<<<1, 256, 0, s>>>(z.part, z.nblk_b, dV, z.nrm, betas + j);
    GATO_LAUNCH_TRY();
    k_beta_scale<T><<<grid_for(n / (16 / (int64_t)sizeof(T)) + 1, 256), 256, 0, s>>>(W, n, z.nrm);
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  const size_t smt = (size_t)(kLzThreads / 32) * nk * sizeof(double);
  const size_t smn = (size_t)nk * sizeof(double);
  if (smt > 48 * 1024)
    GATO_TRY(raise_smem_limit(reinterpret_cast<const void*>(k_gemv_t<T, T>), smt));
  // alpha_j = dV <v_j, w'>
  k_gemv_t<T, T><<<z.nblk_t, kLzThreads, (kLzThreads / 32) * sizeof(double), s>>>(vj, n, 1, W, p1, n,
                                                                                  z.part);
  GATO_LAUNCH_TRY();
  GATO_TRY(finalize_sums(z.part, 1, z.nblk_t, dV, alphas + j, s));
  Pre<T> p2 = p1;
  p2.u[1] = vj;
  p2.s[1] = alphas + j;
  for (int p = 0; p < passes; ++p) {
    const Pre<T>& pp = p == 0 ? p2 : Pre<T>();
    k_gemv_t<T, T><<<z.nblk_t, kLzThreads, smt, s>>>(Vb, n, nk, W, pp, n, z.part);
    GATO_LAUNCH_TRY();
    GATO_TRY(finalize_sums(z.part, nk, z.nblk_t, dV, z.coef, s));
    k_gemv_n<T, float><<<z.nblk, kLzThreads, smn, s>>>(Vb, n, nk, W, pp, z.coef, n, z.part);
    GATO_LAUNCH_TRY();
  }
  k_beta_finalize<<<1, 256, 0, s>>>(z.part, z.nblk, dV, z.nrm, betas + j);
  GATO_LAUNCH_TRY();
  k_beta_scale<T><<<grid_for(n / (16 / (int64_t)sizeof(T)) + 1, 256), 256, 0, s>>>(W, n, z.nrm);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

template <typename T>
int lz_finish(const T* Vb, int64_t n, int m, int K, double tol, const double* alphas,
              const double* betas, double* evals, T* evecs, int* flag, const LzScratch& z,
              cudaStream_t s) {
  const size_t sme = (size_t)10 * m * sizeof(double);
  if (sme > 227 * 1024)
    return fail(GATO_EUNSUPPORTED, "lanczos: m = %d exceeds the tridiagonal eigensolver's shared memory", m);
  if (sme > 48 * 1024)
    GATO_TRY(raise_smem_limit(reinterpret_cast<const void*>(k_tridiag_eig), sme));
  k_tridiag_eig<<<K, 32, sme, s>>>(alphas, betas, m, K, evals, z.work, device_error_word());
  GATO_LAUNCH_TRY();
  k_tridiag_finish<<<1, 32, 0, s>>>(alphas, betas, m, K, evals, z.work, evals, z.Y, flag, tol);
  GATO_LAUNCH_TRY();
  constexpr int KB = 4;
  const size_t smr = (size_t)KB * m * sizeof(T);
  if (smr > 48 * 1024)
    GATO_TRY(raise_smem_limit(reinterpret_cast<const void*>(k_ritz<T, KB>), smr));
  for (int k0 = 0; k0 < K; k0 += KB) {
    k_ritz<T, KB><<<grid_for(n, 256, 152 * 8), 256, smr, s>>>(Vb, n, m, z.Y, k0, K, evecs, n);
    GATO_LAUNCH_TRY();
  }
  return GATO_OK;
}

// ---- one basis sweep per step (FP32 basis) ------------------------------------------
// The classical Gram-Schmidt step above reads the basis twice: once for the
// coefficients c = V^T w'' and once for the correction w'' - V c. Here the
// operator is applied to the uncorrected three-term vector
//   w^_j = F v_j - beta_{j-1} v_{j-1} - alpha_j v_j,
// and the sweep of step j+1 recovers both the new basis vector and its image,
//   v_{j+1}   = (w^_j - V_j c_j) / beta_j,
//   F v_{j+1} = (F w^_j - F V_j c_j) / beta_j,  F V_j c_j = V_{j+1} g,  g = T~ c_j,
// from the Lanczos relation F v_k = beta_{k-1} v_{k-1} + alpha_k v_k + beta_k v_{k+1}
// + V_k c_k, which holds for the computed quantities to rounding (T~ is the
// upper Hessenberg matrix of alpha, beta and every earlier c). The same sweep
// forms the projections of the next step from the identity
//   c_{j+1,k} = <v_k, F v_{j+1}> - beta_j <v_k, v_j> - alpha_{j+1} <v_k, v_{j+1}>,
// taking <v_k, v_j> from the previous sweep. So each step reads the basis once
// (plus four vectors), where the two-sweep form reads it twice; in exact
// arithmetic both give the reference's v, alpha and beta. beta_j comes from
// |w^_j|^2 - |c_j|^2 (Pythagoras; the c_j are the small reorthogonalisation
// coefficients), |w^_j|^2 summed in float-float when w^_j is formed.
//
// Sweep kernel: persistent blocks walk chunks of 64-256 elements; a producer
// warp stages rows v_0..v_{j-1} of a chunk (one 2-D TMA box), w^ and F w^ (two
// 1-D bulk copies) into a ring of shared buffers (full/empty mbarriers,
// bounded waits); the consumers form v_j and F v_j of the chunk (256 / width
// threads per element, each over a share of the basis), write them out and
// keep them as two more rows, and 1-8 threads per basis vector k accumulate
// <v_k, F v_j> and <v_k, v_j> over their chunks (FP32 per chunk, FP64 across
// chunks). Chunk width, ring depth and blocks per SM follow j (fz_ce,
// fz_stages). Only the FP32 basis takes this path: FP64 products would make
// the sweep FP64-bound on GB300. After each sweep, k_fz_form sums the block
// partials (one warp per row), forms alpha_j, the next correction row and w^_j;
// k_fz_post2 forms beta_j and the next sweep's coefficients on the run's own
// side stream while the operator is applied to w^_j.
constexpr int kFzCE = 128;                  // the middle chunk width; n must be a multiple
constexpr int kFzWarps = 8;                 // consumer warps
constexpr int kFzThreads = 32 * (kFzWarps + 1);
constexpr int kFzMaxM = 200;                // basis rows + 4 of a chunk, two buffers, fit in shared memory

__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Named barrier over n threads that also ORs a predicate: every participant gets the same answer.
__device__ __forceinline__ bool named_sync_or(int id, int n, bool v) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 q, %3, 0;\n\tbar.red.or.pred p, %1, %2, q;\n\t"
      "selp.s32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"(id), "r"(n), "r"((int)v)
      : "memory");
  return r != 0;
}

// Chunk width of a step-j sweep: 256 elements while the basis is short (fewer, larger chunks
// amortise the per-chunk latency), 128 while two blocks' staging fits one SM (j <= 98), then 64
// (measured at 128^3: 64-wide chunks lose to 128 below j = 100 and win above). The element count
// must divide into chunks (n % 256 == 0 for the widest).
__host__ __device__ constexpr int fz_ce(int j, int64_t n) {
  return (j < 32 && n % 256 == 0) ? 256 : (j < 99 ? 128 : 64);
}
// Threads per projection row in phase B: as many as keep (j + 1) rows within the 256 consumers.
__host__ __device__ constexpr int fz_tpk(int j) { return j < 32 ? 8 : (j < 64 ? 4 : (j < 128 ? 2 : 1)); }
// Staged row width (floats): the chunk plus a pad that makes the 16-byte reads of one phase-B
// phase (8 threads: 8 / tpk rows, tpk consecutive vectors each) fall in 8 distinct 4-bank groups:
// the row stride is 4 tpk words mod 32. The staging copy's box is this wide (the extra columns are
// the next chunk's, or zero past the end of the vector).
__host__ __device__ constexpr int fz_rw(int j, int ce) { return fz_tpk(j) == 8 ? ce : ce + 4 * fz_tpk(j); }
// floats per staging buffer: j + 4 rows, rounded up to 128 bytes (TMA destinations)
__host__ __device__ constexpr int fz_bufstride(int j, int ce) {
  return ((j + 4) * fz_rw(j, ce) * 4 + 127) / 128 * 32;
}

constexpr int kFzMaxStages = 32;   // small-j chunks are a few KB: many in flight per SM
constexpr size_t kFzFixed = 2 * (kFzMaxM + 2) * sizeof(float) + 4 * kFzCE * sizeof(float) +
                            2 * kFzMaxStages * sizeof(uint64_t) + 128;
constexpr size_t kFzSmemCap = 220 * 1024;
__host__ __device__ constexpr size_t fz_smem(int j, int ce, int nst) {
  return (size_t)nst * fz_bufstride(j, ce) * sizeof(float) + kFzFixed;
}
// Staging depth of a step-j sweep: as many buffers as let two blocks share an SM (the two blocks
// hide each other's per-chunk latency), else as many as one block can hold (at least two).
inline int fz_stages(int j, int ce) {
  const size_t half = 113 * 1024 - kFzFixed;   // two blocks and their reserved shared memory per SM
  const int n2 = (int)(half / (fz_bufstride(j, ce) * sizeof(float)));
  if (n2 >= 2) return n2 < kFzMaxStages ? n2 : kFzMaxStages;
  const int nst = (int)((kFzSmemCap - kFzFixed) / (fz_bufstride(j, ce) * sizeof(float)));
  return nst < kFzMaxStages ? nst : kFzMaxStages;
}

// j: this sweep forms v_j (basis slot j) and u_j = F v_j (U). wh: w^_{j-1}; z: F w^_{j-1};
// c (j entries), g (j + 1 entries), binv = {beta_{j-1}, 1 / beta_{j-1}}. part: [2][j+1][grid].
// tv: the basis as a 2-D tensor {n, slots} with a {fz_rw(j), j} box: one copy stages rows
// v_0..v_{j-1} of a chunk in the padded row layout the sweep reads.
// At most 96 registers, so two blocks (18 warps) fit one SM's register file.
__global__ void __maxnreg__(96)
    k_fz_sweep(const __grid_constant__ CUtensorMap tv, float* V, int64_t n, int j, int CE, int NST, const float* wh,
               const float* z, float* U, const double* c, const double* g, const double* binv, double* part,
               int* err) {
  extern __shared__ __align__(128) unsigned char fzs[];
  unsigned char* base = fzs + ((128u - (smem_u32(fzs) & 127u)) & 127u);
  float* buf0 = reinterpret_cast<float*>(base);
  const int BS = fz_bufstride(j, CE), RW = fz_rw(j, CE), TPK = fz_tpk(j);   // NST staging buffers
  // (c_k, g_k) pairs, rounded once to FP32: one 8-byte shared load per basis row in phase A
  float2* csg = reinterpret_cast<float2*>(buf0 + (size_t)NST * BS);
  float* pa = reinterpret_cast<float*>(csg + (kFzMaxM + 2));   // [2][P-1][CE]: the other groups' partial corrections
  uint64_t* full = reinterpret_cast<uint64_t*>(pa + 4 * kFzCE);   // pa holds up to 2 x 3 x 64 floats
  uint64_t* empty = full + kFzMaxStages;
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nch = n / CE;
  if (threadIdx.x == 0) {
    for (int b = 0; b < NST; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], kFzWarps);
    }
    abort_flag = 0;
    fence_barrier_init();
  }
  for (int k = threadIdx.x; k <= j; k += blockDim.x) csg[k] = make_float2(k < j ? (float)c[k] : 0.f, (float)g[k]);
  __syncthreads();
  if (warp == kFzWarps) {   // producer
    if (lane == 0) {
      int it = 0;
      for (int64_t ch = blockIdx.x; ch < nch; ch += gridDim.x, ++it) {
        const int b = it % NST;
        if (it >= NST && !mbar_wait_bounded(&empty[b], (uint32_t)(((it / NST) - 1) & 1), err, 115)) {
          *abort_v = 1;
          break;
        }
        if (*abort_v) break;
        float* bf = buf0 + (size_t)b * BS;
        const int64_t off = ch * CE;
        const uint32_t RB = (uint32_t)CE * sizeof(float);
        mbar_expect_tx(&full[b], (uint32_t)j * RW * sizeof(float) + 2 * RB);
        if (j > 0) tma_load_2d(bf, &tv, &full[b], (int)off, 0);
        bulk_load(bf + (size_t)(j + 2) * RW, wh + off, RB, &full[b]);
        bulk_load(bf + (size_t)(j + 3) * RW, z + off, RB, &full[b]);
      }
      if (*abort_v)   // copies in flight land (bounded) before the block exits
        for (int p = it > NST ? it - NST : 0; p < it; ++p)
          mbar_wait_bounded(&full[p % NST], (uint32_t)((p / NST) & 1), err, 116);
    }
    return;
  }
  // consumers
  const int t = threadIdx.x;
  // phase A: element e of the chunk, group h of P = 256 / CE splitting the basis rows
  const int P = 256 / CE;
  const int e = t % CE, h = t / CE;
  const int k0 = (int)((int64_t)j * h / P), k1 = (int)((int64_t)j * (h + 1) / P);
  const int kb = t / TPK, sub = t % TPK;       // phase B: projection row kb, part sub of the chunk
  const float bi = (float)binv[1];
  const float gj = csg[j].y;
  double accA = 0.0, accD = 0.0;
  int it = 0;
  bool ok = true;
  for (int64_t ch = blockIdx.x; ch < nch; ch += gridDim.x, ++it) {
    const int b = it % NST;
    // one decision for every consumer: the producer may raise the flag at any moment
    bool bad = *abort_v != 0;
    if (!bad) bad = !mbar_wait_bounded(&full[b], (uint32_t)((it / NST) & 1), err, 117);
    if (named_sync_or(1, kFzWarps * 32, bad)) {
      if (t == 0) {
        *abort_v = 1;   // the producer stops issuing
        // this chunk's copies land (bounded) before the block can leave
        mbar_wait_bounded(&full[b], (uint32_t)((it / NST) & 1), err, 118);
      }
      ok = false;
      break;
    }
    float* bf = buf0 + (size_t)b * BS;
    // phase A: corrections of this half of the basis, two accumulator pairs
    float cv0 = 0.f, cu0 = 0.f, cv1 = 0.f, cu1 = 0.f;
    int k = k0;
#pragma unroll 4
    for (; k + 1 < k1; k += 2) {
      const float x0 = bf[(size_t)k * RW + e], x1 = bf[(size_t)(k + 1) * RW + e];
      const float2 a0 = csg[k], a1 = csg[k + 1];
      cv0 = fmaf(a0.x, x0, cv0);
      cu0 = fmaf(a0.y, x0, cu0);
      cv1 = fmaf(a1.x, x1, cv1);
      cu1 = fmaf(a1.y, x1, cu1);
    }
    if (k < k1) {
      const float x0 = bf[(size_t)k * RW + e];
      const float2 a0 = csg[k];
      cv0 = fmaf(a0.x, x0, cv0);
      cu0 = fmaf(a0.y, x0, cu0);
    }
    float cv = cv0 + cv1, cu = cu0 + cu1;
    if (h > 0) {
      pa[(h - 1) * CE + e] = cv;
      pa[(P - 1 + h - 1) * CE + e] = cu;
    }
    named_sync(1, kFzWarps * 32);
    const int64_t gi = ch * CE + e;
    if (h == 0) {
      for (int q = 1; q < P; ++q) {   // groups in order
        cv += pa[(q - 1) * CE + e];
        cu += pa[(P - 1 + q - 1) * CE + e];
      }
      const float vj = (bf[(size_t)(j + 2) * RW + e] - cv) * bi;
      const float uj = (bf[(size_t)(j + 3) * RW + e] - cu - gj * vj) * bi;
      bf[(size_t)j * RW + e] = vj;
      bf[(size_t)(j + 1) * RW + e] = uj;
      V[(int64_t)j * n + gi] = vj;
      U[gi] = uj;
    }
    named_sync(1, kFzWarps * 32);
    // phase B: the TPK threads of row kb <= j accumulate <v_kb, u_j> and <v_kb, v_j> over the
    // chunk's 16-byte vectors sub, sub + TPK, ..., then reduce across those lanes
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), d = a;
    if (kb <= j) {
      const float4* rk = reinterpret_cast<const float4*>(bf + (size_t)kb * RW);
      const float4* ru = reinterpret_cast<const float4*>(bf + (size_t)(j + 1) * RW);
      const float4* rv = reinterpret_cast<const float4*>(bf + (size_t)j * RW);
#pragma unroll 4
      for (int i = sub; i < CE / 4; i += TPK) {
        const float4 x = rk[i], u = ru[i], v = rv[i];
        a.x = fmaf(x.x, u.x, a.x);
        a.y = fmaf(x.y, u.y, a.y);
        a.z = fmaf(x.z, u.z, a.z);
        a.w = fmaf(x.w, u.w, a.w);
        d.x = fmaf(x.x, v.x, d.x);
        d.y = fmaf(x.y, v.y, d.y);
        d.z = fmaf(x.z, v.z, d.z);
        d.w = fmaf(x.w, v.w, d.w);
      }
    }
    float sa = (a.x + a.y) + (a.z + a.w), sd = (d.x + d.y) + (d.z + d.w);
    for (int o = TPK / 2; o > 0; o >>= 1) {   // TPK consecutive lanes of one warp
      sa += __shfl_xor_sync(0xffffffffu, sa, o);
      sd += __shfl_xor_sync(0xffffffffu, sd, o);
    }
    if (kb <= j && sub == 0) {
      accA += (double)sa;
      accD += (double)sd;
    }
    fence_proxy_async_smem();   // the chunk's reads and writes of bf precede the next copy into it
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
  if (ok && kb <= j && sub == 0) {
    const int G = gridDim.x;
    part[(int64_t)kb * G + blockIdx.x] = accA;
    part[(int64_t)(j + 1 + kb) * G + blockIdx.x] = accD;
  }
}

// w^_j = u_j - beta_{j-1} v_{j-1} - alpha_j v_j (field type products) and its float-float |.|^2 partials,
// with the sweep's projections reduced on the way in. part holds the sweep's block partials, rows
// r <= j for a_k = dV <v_k, u_j> and rows j + 1 + k for d_k = dV <v_k, v_j>; a row sum is one warp
// (lanes stride the G partials, then a fixed-order tree), the same sum wherever it runs. Every block
// forms alpha_j = a_j - beta_{j-1} b_j (b_j = d_{j-1}); warps spread over the blocks form row j of Cm,
// c_k = a_k - beta_{j-1} b_k - alpha_j d_k (b_k = <v_k, v_{j-1}> from the previous sweep for k < j,
// d_{j-1} for k = j), and dprev <- d; block 0 records alpha_j.
__global__ void k_fz_form(const float* __restrict__ U, const float* __restrict__ vm1, const float* __restrict__ vj,
                          float* wh, int64_t n, const double* part, int G, double dV, double* alphas,
                          const double* betas, double* dprev, double* Cm, int m, int j, double* partn) {
  __shared__ double sh[32];
  __shared__ double s_ad[2];   // a_j, d_{j-1}
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  auto rowsum = [&](int r) {
    double v = 0.0;
    for (int q = lane; q < G; q += 32) v += part[(int64_t)r * G + q];
    return warp_sum(v) * dV;
  };
  if (warp == 0) {
    const double aj = rowsum(j);
    const double dj1 = j > 0 ? rowsum(2 * j) : 0.0;
    if (lane == 0) {
      s_ad[0] = aj;
      s_ad[1] = dj1;
    }
  }
  __syncthreads();
  const double beta = j > 0 ? betas[j - 1] : 0.0;
  const double ald = s_ad[0] - beta * s_ad[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) alphas[j] = ald;
  for (int k = blockIdx.x * nw + warp; k <= j; k += gridDim.x * nw) {
    const double sak = rowsum(k), sdk = rowsum(j + 1 + k);
    if (lane == 0) {
      // the lane reads dprev[k] before it overwrites the same entry: no other thread touches it
      const double bk = j == 0 ? 0.0 : (k < j ? dprev[k] : s_ad[1]);
      Cm[(int64_t)j * m + k] = sak - beta * bk - ald * sdk;
      dprev[k] = sdk;
    }
  }
  const float be = (float)beta, al = (float)ald;
  Acc<float> acc;
  const int64_t nv = n / 4;
  const float4* U4 = reinterpret_cast<const float4*>(U);
  const float4* A4 = reinterpret_cast<const float4*>(j > 0 ? vm1 : vj);
  const float4* B4 = reinterpret_cast<const float4*>(vj);
  float4* W4 = reinterpret_cast<float4*>(wh);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 u = U4[i], a = A4[i], b = B4[i];
    float4 w;
    w.x = u.x - be * a.x - al * b.x;
    w.y = u.y - be * a.y - al * b.y;
    w.z = u.z - be * a.z - al * b.z;
    w.w = u.w - be * a.w - al * b.w;
    W4[i] = w;
    acc.add_prod(w.x, w.x);
    acc.add_prod(w.y, w.y);
    acc.add_prod(w.z, w.z);
    acc.add_prod(w.w, w.w);
  }
  const double v = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) partn[blockIdx.x] = v;
}

// beta_j = sqrt(dV |w^_j|^2 - |c_j|^2), binv = {beta_j, 1 / beta_j or 0}, and the next sweep's
// c = c_j and g_i = sum_k T~_{ik} c_k, i <= j + 1. Every block forms beta_j from the same sums in
// the same order (so all hold the same bits) and one warp per g_i sums its column of Cm across the
// lanes; block 0 writes beta_j, binv and c. Launched with kFzPost2Threads threads per block.
constexpr int kFzPost2Threads = 256;
__global__ void __launch_bounds__(kFzPost2Threads)
    k_fz_post2(const double* part, int nb, double dV, const double* Cm, int m, int j, const double* alphas,
               double* betas, double* binv, double* c_next, double* g_next) {
  __shared__ double sh[32];
  __shared__ double sc[kFzMaxM + 1];
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += part[i];
  const double wn = block_sum(v, sh);
  double c2 = 0.0;
  for (int k = threadIdx.x; k <= j; k += blockDim.x) {
    const double ck = Cm[(int64_t)j * m + k];
    sc[k] = ck;
    c2 += ck * ck;
  }
  const double cn = block_sum(c2, sh);   // its barriers also publish sc
  const double b2 = wn * dV - cn;
  const double beta = b2 > 0.0 ? sqrt(b2) : 0.0;
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) {
      betas[j] = beta;
      binv[0] = beta;
      binv[1] = beta > 0.0 ? 1.0 / beta : 0.0;
    }
    for (int k = threadIdx.x; k <= j; k += blockDim.x) c_next[k] = sc[k];
  }
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i > j + 1) return;
  double gi = 0.0;
  for (int k = i + lane; k <= j; k += 32) gi += sc[k] * Cm[(int64_t)k * m + i];
  gi = warp_sum(gi);
  if (lane == 0) {
    // the tridiagonal part of T~ row i: beta_i c_{i+1} + alpha_i c_i + beta_{i-1} c_{i-1}
    if (i + 1 <= j) gi += sc[i + 1] * betas[i];
    if (i <= j) gi += sc[i] * alphas[i];
    if (i >= 1) gi += sc[i - 1] * (i - 1 == j ? beta : betas[i - 1]);
    g_next[i] = gi;
  }
}

struct FzScratch {
  float *wh, *z, *u;
  double *Cm, *dprev, *c, *g, *binv, *part, *partn;
  int grid, nbf, sms;   // grid: the most sweep blocks of any step
};

int fz_scratch(cudaStream_t s, int64_t n, int m, FzScratch& f) {
  int dev = 0, sms = 0;
  GATO_CUDA_TRY(cudaGetDevice(&dev));
  GATO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  f.sms = sms;
  f.grid = (int)std::min<int64_t>(n / 64, 4 * (int64_t)sms);
  f.nbf = (int)std::min<int64_t>((n / 4 + 255) / 256, 4 * sms);
  const size_t vec = (size_t)n * sizeof(float);
  const size_t dbl = (size_t)m * m + m + (m + 1) + (m + 2) + 2 + (size_t)2 * (m + 1) * f.grid + f.nbf;
  unsigned char* p = (unsigned char*)stream_scratch(s, 3 * vec + dbl * sizeof(double) + 256, kSlotLanczosSweep);
  if (!p) return fail(GATO_ENOMEM, "lanczos: sweep scratch allocation failed");
  f.wh = (float*)p;
  f.z = f.wh + n;
  f.u = f.z + n;
  double* d = (double*)(p + 3 * vec);
  f.Cm = d;
  f.dprev = f.Cm + (size_t)m * m;
  f.c = f.dprev + m;
  f.g = f.c + (m + 1);
  f.binv = f.g + (m + 2);
  f.part = f.binv + 2;
  f.partn = f.part + (size_t)2 * (m + 1) * f.grid;
  return GATO_OK;
}

std::atomic<int> g_lz_sweeps{1};   // 1: one basis sweep per step where supported, 2: two

bool fz_ok(const float* Vb, int64_t n, int m, int passes) {
  return g_lz_sweeps.load() == 1 && passes == 1 && m <= kFzMaxM && n % kFzCE == 0 && n / kFzCE >= 1 &&
         ((uintptr_t)Vb % 16) == 0;
}

__global__ void k_fz_init(double* g, double* binv) {
  g[0] = 0.0;
  binv[0] = 1.0;
  binv[1] = 1.0;
}

// A stream of the Lanczos run's own, with the two events that fork work onto it and join it back
// (released on every exit; pending work finishes first).
struct FzSide {
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int create() {
    GATO_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    GATO_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    GATO_CUDA_TRY(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
    return GATO_OK;
  }
  ~FzSide() {
    if (join) cudaEventDestroy(join);
    if (fork) cudaEventDestroy(fork);
    if (st) cudaStreamDestroy(st);
  }
};

int lanczos_fused(gato_operator& op, const void* psi0, int m, int K, double tol, float* Vb, double* evals,
                  float* evecs, double* alphas, double* betas, int* flag, cudaStream_t s) {
  const int64_t n = op_n3(op);
  const double dV = op.dV;
  LzScratch z;
  GATO_TRY(lz_scratch(s, n, m, K, z, false));
  FzScratch f;
  GATO_TRY(fz_scratch(s, n, m, f));
  GATO_TRY(lz_begin<float>(psi0, Vb, n, dV, z, s));
  GATO_TRY(op_apply(op, Vb, f.z, s));   // F v_0
  k_fz_init<<<1, 1, 0, s>>>(f.g, f.binv);
  GATO_LAUNCH_TRY();
  GATO_TRY(raise_smem_limit(reinterpret_cast<const void*>(k_fz_sweep), kFzSmemCap));
  if (n > INT32_MAX) return fail(GATO_EUNSUPPORTED, "lanczos: field too large for the sweep's tensor map");
  FzSide side;
  GATO_TRY(side.create());
  for (int j = 0; j < m; ++j) {
    const float* wh = j == 0 ? Vb : f.wh;   // v_0 itself (beta = 1, c = g = 0) at the first step
    const int ce = fz_ce(j, n);
    alignas(64) unsigned char tm[128];
    TmaBox bx;
    bx.rank = 2;
    bx.dims[0] = (uint64_t)n;
    bx.dims[1] = (uint64_t)m + 1;
    bx.strides_bytes[0] = (uint64_t)n * sizeof(float);
    bx.box[0] = (uint32_t)fz_rw(j, ce);
    bx.box[1] = j > 0 ? (uint32_t)j : 1u;   // unused at j = 0
    GATO_TRY(encode_tma(tm, GATO_F32, Vb, bx));
    const int nst = fz_stages(j, ce);
    const size_t smj = fz_smem(j, ce, nst);
    static std::atomic<int> per_sm_of[kFzMaxM];   // resident sweep blocks per SM, by step (0: unknown)
    int per_sm = per_sm_of[j].load();
    if (per_sm == 0) {
      GATO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fz_sweep, kFzThreads, smj));
      if (per_sm < 1) return fail(GATO_EUNSUPPORTED, "lanczos: sweep block does not fit");
      per_sm_of[j].store(per_sm);
    }
    const int G = (int)std::min<int64_t>(std::min<int64_t>(n / ce, (int64_t)std::min(per_sm, 4) * f.sms),
                                         f.grid);
    k_fz_sweep<<<G, kFzThreads, smj, s>>>(*reinterpret_cast<const CUtensorMap*>(tm), Vb, n, j, ce, nst, wh, f.z,
                                          f.u, f.c, f.g, f.binv, f.part, device_error_word());
    GATO_LAUNCH_TRY();
    k_fz_form<<<f.nbf, 256, 0, s>>>(f.u, j > 0 ? Vb + (int64_t)(j - 1) * n : nullptr, Vb + (int64_t)j * n, f.wh, n,
                                    f.part, G, dV, alphas, betas, f.dprev, f.Cm, m, j, f.partn);
    GATO_LAUNCH_TRY();
    // beta_j and the next sweep's coefficients on the side stream, beside the operator apply to w^_j
    // (which reads neither); the next sweep, and the eigensolve after the last step, wait for them
    GATO_CUDA_TRY(cudaEventRecord(side.fork, s));
    GATO_CUDA_TRY(cudaStreamWaitEvent(side.st, side.fork, 0));
    constexpr int gpb = kFzPost2Threads / 32;   // g_i per block
    k_fz_post2<<<(j + 2 + gpb - 1) / gpb, kFzPost2Threads, 0, side.st>>>(f.partn, f.nbf, dV, f.Cm, m, j, alphas,
                                                                          betas, f.binv, f.c, f.g);
    GATO_LAUNCH_TRY();
    GATO_CUDA_TRY(cudaEventRecord(side.join, side.st));
    if (j + 1 < m) GATO_TRY(op_apply(op, f.wh, f.z, s));
    GATO_CUDA_TRY(cudaStreamWaitEvent(s, side.join, 0));
  }
  return lz_finish<float>(Vb, n, m, K, tol, alphas, betas, evals, evecs, flag, z, s);
}

template <typename T>
int lanczos_typed(gato_operator& op, const void* psi0, int m, int K, double tol, int passes,
                  void* krylov, double* evals, void* evecs, double* alphas, double* betas,
                  int* flag, cudaStream_t s) {
  const int64_t n = op_n3(op);
  T* Vb = (T*)krylov;
  if constexpr (sizeof(T) == 4) {
    if (fz_ok(Vb, n, m, passes))
      return lanczos_fused(op, psi0, m, K, tol, Vb, evals, (float*)evecs, alphas, betas, flag, s);
  }
  LzScratch z;
  GATO_TRY(lz_scratch(s, n, m, K, z, sizeof(T) == 8));
  GATO_TRY(lz_begin<T>(psi0, Vb, n, op.dV, z, s));
  for (int j = 0; j < m; ++j) {
    GATO_TRY(op_apply(op, Vb + (int64_t)j * n, Vb + (int64_t)(j + 1) * n, s));
    GATO_TRY(lz_step<T>(Vb, n, op.dV, j, passes, alphas, betas, z, s));
  }
  return lz_finish<T>(Vb, n, m, K, tol, alphas, betas, evals, (T*)evecs, flag, z, s);
}

}  // namespace

}  // namespace gato

using namespace gato;

extern "C" int gato_lanczos(gato_op_t op, const void* psi0, int m, int K, double tol,
                            int reorth_passes, void* krylov, double* evals_dev, void* evecs,
                            double* alphas_dev, double* betas_dev, int* flag_dev, void* stream) {
  if (!op || !psi0 || !krylov || !evals_dev || !evecs || !alphas_dev || !betas_dev || !flag_dev)
    return fail(GATO_EBADARG, "gato_lanczos: NULL argument");
  if (m < 1 || K < 1 || K > m) return fail(GATO_EBADARG, "gato_lanczos: need 1 <= K <= m (m=%d K=%d)", m, K);
  if (K > 1024) return fail(GATO_EUNSUPPORTED, "gato_lanczos: at most 1024 eigenpairs");
  if (reorth_passes < 1 || reorth_passes > 2) return fail(GATO_EBADARG, "reorth_passes must be 1 or 2");
  cudaStream_t s = as_stream(stream);
  if (op->dtype == GATO_F64)
    return lanczos_typed<double>(*op, psi0, m, K, tol, reorth_passes, krylov, evals_dev, evecs,
                                 alphas_dev, betas_dev, flag_dev, s);
  return lanczos_typed<float>(*op, psi0, m, K, tol, reorth_passes, krylov, evals_dev, evecs,
                              alphas_dev, betas_dev, flag_dev, s);
}

extern "C" int gato_lanczos_begin(int dtype, int64_t n, double dV, const void* psi0, void* krylov,
                                  int m, int K, void* stream) {
  if (!psi0 || !krylov || n < 1 || m < 1 || K < 1 || K > m) return fail(GATO_EBADARG, "gato_lanczos_begin: bad arguments");
  cudaStream_t s = as_stream(stream);
  LzScratch z;
  GATO_TRY(lz_scratch(s, n, m, K, z, dtype == GATO_F64));
  if (dtype == GATO_F64) return lz_begin<double>(psi0, (double*)krylov, n, dV, z, s);
  return lz_begin<float>(psi0, (float*)krylov, n, dV, z, s);
}

extern "C" int gato_lanczos_step(int dtype, int64_t n, double dV, void* krylov, int j, int m, int K,
                                 int reorth_passes, double* alphas_dev, double* betas_dev,
                                 void* stream) {
  if (!krylov || !alphas_dev || !betas_dev || j < 0 || j >= m) return fail(GATO_EBADARG, "gato_lanczos_step: bad arguments");
  if (reorth_passes < 1 || reorth_passes > 2) return fail(GATO_EBADARG, "reorth_passes must be 1 or 2");
  cudaStream_t s = as_stream(stream);
  LzScratch z;
  GATO_TRY(lz_scratch(s, n, m, K, z, dtype == GATO_F64));
  if (dtype == GATO_F64) return lz_step<double>((double*)krylov, n, dV, j, reorth_passes, alphas_dev, betas_dev, z, s);
  return lz_step<float>((float*)krylov, n, dV, j, reorth_passes, alphas_dev, betas_dev, z, s);
}

extern "C" int gato_lanczos_finish(int dtype, int64_t n, const void* krylov, int m, int K, double tol,
                                   const double* alphas_dev, const double* betas_dev,
                                   double* evals_dev, void* evecs, int* flag_dev, void* stream) {
  if (!krylov || !alphas_dev || !betas_dev || !evals_dev || !evecs || !flag_dev || m < 1 || K < 1 || K > m)
    return fail(GATO_EBADARG, "gato_lanczos_finish: bad arguments");
  cudaStream_t s = as_stream(stream);
  LzScratch z;
  GATO_TRY(lz_scratch(s, n, m, K, z, dtype == GATO_F64));
  if (dtype == GATO_F64)
    return lz_finish<double>((const double*)krylov, n, m, K, tol, alphas_dev, betas_dev, evals_dev, (double*)evecs, flag_dev, z, s);
  return lz_finish<float>((const float*)krylov, n, m, K, tol, alphas_dev, betas_dev, evals_dev, (float*)evecs, flag_dev, z, s);
}

// Tuning (no reference counterpart): sweeps of the basis per Lanczos step on the FP32 path,
// 1 (the one-sweep form, where m <= 200 and n is a multiple of 128) or 2 (classical
// Gram-Schmidt: coefficient sweep, then correction sweep).
extern "C" int gato_lanczos_tune(int sweeps) {
  if (sweeps != 1 && sweeps != 2) return fail(GATO_EBADARG, "gato_lanczos_tune: sweeps must be 1 or 2");
  g_lz_sweeps.store(sweeps);
  return GATO_OK;
}
