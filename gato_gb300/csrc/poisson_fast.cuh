// Pair-solve pipeline kernels on the register-resident two-pass FFT engine
// (fft2.cuh), one instantiation per supported doubled-grid size M.
#pragma once
#include <atomic>
#include "fft2.cuh"
#include "poisson.cuh"
#include "ptx.cuh"

namespace gato {
namespace fast {

using namespace fft2;


// The COUNT-entry stage-twiddle table split into a register prefetch at
// kernel entry and a shared-memory store placed after the kernel's own field
// loads are issued, so the two global latencies overlap instead of adding up.
template <typename T2, int COUNT, int NT>
struct TwPrefetch {
  static constexpr int K = (COUNT + NT - 1) / NT;
  T2 v[K];
  __device__ __forceinline__ explicit TwPrefetch(const T2* tw) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = threadIdx.x + k * NT;
      if (i < COUNT) v[k] = tw[i];
    }
  }
  __device__ __forceinline__ void store(T2* tws) const {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int i = threadIdx.x + k * NT;
      if (i < COUNT) tws[i] = v[k];
    }
  }
};

// Strided-line passes (y forward, x forward * kernel * x inverse, y inverse).
// FULL: every CTA has L real columns (ncols % L == 0), so no per-access guard.
template <typename T, int R1, int R2, int L, int MODE, bool FULL>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_cols(const typename Cplx<T>::type* in, typename Cplx<T>::type* out, ColGeom g,
           const typename Cplx<T>::type* tw, const T* ghat, int H) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, LP = L + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + M * LP;
  const TwPrefetch<T2, R1 * TwRow<T2, R2>::S, L * Shape<R1, R2>::RMAX> twp(tw);
  const int outer = blockIdx.x, col0 = blockIdx.y * L, f = blockIdx.z;
  const int t = threadIdx.x;
  const int line = t % L, q = t / L;   // q: n2 in stages 1/B, k1 in stages 2/A
  const bool live = FULL || line < g.ncols - col0;
  // per-thread bases: element (pos, line) of this CTA's tile is base[pos * ps]
  const T2* src = in + f * g.in_fs + outer * g.in_os + col0 + line;
  T2* dst = out + f * g.out_fs + outer * g.out_os + col0 + line;
  const int64_t ips = g.in_ps, ops = g.out_ps;
  T2 X[R2];
  if (MODE != COL_INV) {
    if (q < R2) {
      const T2* b1 = src + q * ips;
      fwd_stage1<T2, R1, R2, true>(buf, LP, line, q, [&](int pos) {
        T2 v;
        if (live) v = b1[(pos - q) * ips];   // pos - q = R2 n1: a compile-time multiple of R2
        else v.x = v.y = 0;
        return v;
      });
    }
    twp.store(tws);
    __syncthreads();
    if (q < R1) fwd_stage2<T2, R1, R2>(buf, LP, line, q, tws, X);
  } else {
    __syncthreads();
    if (q < R1) {
      const T2* b = src + q * ips;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        if (live) X[k2] = b[(int64_t)(R1 * k2) * ips];
        else X[k2].x = X[k2].y = 0;
      }
    }
    twp.store(tws);   // first read in inv_stageA, behind the barrier below
  }
  if (MODE == COL_FWD) {
    if (q < R1 && live) {
      T2* b = dst + q * ops;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) b[(int64_t)(R1 * k2) * ops] = X[k2];
    }
    return;
  }
  if (MODE == COL_FMI && q < R1) {
    static_assert(R2 % 2 == 0, "the octant fold below splits k2 at R2 / 2");
    const int ky = outer, kyo = ky <= M - ky ? ky : M - ky;
    const int kz = col0 + line, kzo = kz <= M - kz ? kz : M - kz;
    const int64_t HH = (int64_t)H * H, st = (int64_t)R1 * HH;
    // kx = q + R1 k2 (q < R1): k2 < R2/2 gives kx <= M/2, read at kx; the upper
    // half folds to M - kx = (M - q) - R1 k2.
    const T* glo = ghat + (int64_t)q * HH + (int64_t)kyo * H + kzo;
    const T* ghi = ghat + (int64_t)(M - q) * HH + (int64_t)kyo * H + kzo;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      const T gv = live ? (k2 < R2 / 2 ? glo[k2 * st] : ghi[-k2 * st]) : (T)0;
      X[k2].x *= gv;
      X[k2].y *= gv;
    }
  }
  __syncthreads();   // stage-2 reads of buf are complete
  if (q < R1) inv_stageA<T2, R1, R2>(buf, LP, line, q, tws, X);
  __syncthreads();
  if (q < R2) {
    T2* b = dst + q * ops;
    inv_stageB<T2, R1, R2, true>(buf, LP, line, q, [&](int pos, T2 v) {
      if (live) b[(pos - q) * ops] = v;
    });
  }
}

// Block sum of a per-thread accumulator, valid in thread 0 only: float-float
// through the shuffles for FP32 (the FP64 pipe is used once per CTA), double
// for FP64. `sh` holds 32 doubles.
__device__ __forceinline__ double block_sum0(const Acc<float>& a, double* sh) {
  FF s = a.s;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float hi = __shfl_xor_sync(0xffffffffu, s.hi, o);
    const float lo = __shfl_xor_sync(0xffffffffu, s.lo, o);
    ff_add(s, hi);
    s.lo += lo;
  }
  float2* shf = reinterpret_cast<float2*>(sh);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) shf[warp] = make_float2(s.hi, s.lo);
  __syncthreads();
  if (threadIdx.x != 0) return 0.0;
  FF t{0.f, 0.f};
  for (int w = 0; w < nw; ++w) {
    ff_add(t, shf[w].x);
    t.lo += shf[w].y;
  }
  return ff_value(t);
}
__device__ __forceinline__ double block_sum0(const Acc<double>& a, double* sh) {
  return block_sum(a.value(), sh);
}

// Energies without the inverse passes (Parseval). The kernel spectrum is
// stored as ghat = G^ dV / M^3, so a part's epilogue energy sum_r rho J with
// J = IDFT(ghat DFT(rho)) (unnormalised) equals sum_k ghat(k) |rho^(k)|^2 over
// the doubled grid (rho is zero outside the N^3 box). For a field F = a + i b
// of two real densities, sum_k ghat |F^|^2 is the sum of both parts' values:
// ghat is real and even, so the cross terms cancel between k and -k. Both
// parts of a field therefore carry one weight and one slot. Each CTA runs the
// x forward transform of its lines of the y-transformed field (as the x pass
// does), sums ghat |X|^2 over its spectrum entries and writes the weighted sum
// to its field's slot, 0 to the other slot.
template <typename T, int R1, int R2, int L, bool FULL>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_cols_fe(const typename Cplx<T>::type* in, ColGeom g, const typename Cplx<T>::type* tw,
              const T* ghat, int H, FeArgs fa) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, LP = L + 1;
  static_assert(R2 % 2 == 0, "the octant fold below splits k2 at R2 / 2");
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sh[32];
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + M * LP;
  const TwPrefetch<T2, R1 * TwRow<T2, R2>::S, L * Shape<R1, R2>::RMAX> twp(tw);
  const int outer = blockIdx.x, col0 = blockIdx.y * L, f = blockIdx.z;
  const int t = threadIdx.x;
  const int line = t % L, q = t / L;
  const bool live = FULL || line < g.ncols - col0;
  const T2* src = in + f * g.in_fs + outer * g.in_os + col0 + line;
  const int64_t ips = g.in_ps;
  if (q < R2) {
    const T2* b1 = src + q * ips;
    fwd_stage1<T2, R1, R2, true>(buf, LP, line, q, [&](int pos) {
      T2 v;
      if (live) v = b1[(pos - q) * ips];
      else v.x = v.y = 0;
      return v;
    });
  }
  twp.store(tws);
  __syncthreads();
  Acc<T> acc;
  if (q < R1) {
    T2 X[R2];
    fwd_stage2<T2, R1, R2>(buf, LP, line, q, tws, X);
    // kx = q + R1 k2, folded into the kernel-spectrum octant as in the x pass
    const int ky = outer, kyo = ky <= M - ky ? ky : M - ky;
    const int kz = col0 + line, kzo = kz <= M - kz ? kz : M - kz;
    const int64_t HH = (int64_t)H * H, st = (int64_t)R1 * HH;
    const T* glo = ghat + (int64_t)q * HH + (int64_t)kyo * H + kzo;
    const T* ghi = ghat + (int64_t)(M - q) * HH + (int64_t)kyo * H + kzo;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      const T gv = live ? (k2 < R2 / 2 ? glo[k2 * st] : ghi[-k2 * st]) : (T)0;
      acc.add_prod(gv, X[k2].x * X[k2].x + X[k2].y * X[k2].y);
    }
  }
  const double s = block_sum0(acc, sh);
  if (t == 0) {
    const int fg = fa.f0 + f;
    const int64_t b = ((int64_t)fg * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const double v = fa.w[fg] * s;
    fa.partials[b] = fa.slot[fg] == 0 ? v : 0.0;
    fa.partials[fa.slot_stride + b] = fa.slot[fg] == 0 ? 0.0 : v;
  }
}

// ---- z passes (rows) ---------------------------------------------------------------
// A CTA owns L consecutive rows (x, y) of the z axis; thread t works on line
// t / RMAX as item j = t % RMAX: n2 in stages 1 and B, k1 in stages 2 and A
// (the RowBuf layout of fft2.cuh). Field rows are read and spectra written
// straight from registers with lanes on consecutive z (or kz), so every
// global access is coalesced and no shared-memory transpose is needed.

// Pair density of part q of a field at element gi (0 when the part is absent).
template <typename T>
__device__ __forceinline__ T part_density(const T* a, const T* b, int64_t gi) {
  if (!a) return (T)0;
  T v = a[gi];
  if (b) v *= b[gi];
  return v;
}

// z forward with the pair-density prologue, one field per CTA (grid.y = field).
template <typename T, int R1, int R2, int L>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_rows_fwd(PassArgs args, int f0, typename Cplx<T>::type* S1, const typename Cplx<T>::type* tw) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, RM = Shape<R1, R2>::RMAX, NT = L * RM;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + L * RowBuf<R1, R2>::LS;
  const TwPrefetch<T2, R1 * TwRow<T2, R2>::S, NT> twp(tw);
  const int p = blockIdx.y;
  const FieldDesc& fd = args.f[f0 + p];
  const int64_t nrows = (int64_t)N * N;
  const int line = threadIdx.x / RM, j = threadIdx.x % RM;
  const int64_t r = (int64_t)blockIdx.x * L + line;
  const bool live = r < nrows;
  // the pair-density factors of the real and imaginary parts (null: factor absent)
  const T* a0 = reinterpret_cast<const T*>(args.in[fd.p[0].a]);
  const T* b0 = fd.p[0].b >= 0 ? reinterpret_cast<const T*>(args.in[fd.p[0].b]) : nullptr;
  const T* a1 = fd.p[1].a >= 0 ? reinterpret_cast<const T*>(args.in[fd.p[1].a]) : nullptr;
  const T* b1 = (a1 && fd.p[1].b >= 0) ? reinterpret_cast<const T*>(args.in[fd.p[1].b]) : nullptr;
  T2 v[R1];
  if (j < R2) {
#pragma unroll
    for (int n1 = 0; n1 < R1 / 2; ++n1) {
      const int64_t gi = r * N + R2 * n1 + j;
      v[n1].x = live ? part_density(a0, b0, gi) : (T)0;
      v[n1].y = live ? part_density(a1, b1, gi) : (T)0;
    }
  }
  twp.store(tws);
  if (j < R2) row_fwd_stage1<T2, R1, R2, true>(buf, line, j, v);
  __syncthreads();
  if (j < R1) {
    T2 X[R2];
    row_fwd_stage2<T2, R1, R2>(buf, line, j, tws, X);
    if (live) {
      T2* d = S1 + (int64_t)p * nrows * M + r * M + j;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) d[R1 * k2] = X[k2];
    }
  }
}

// Padded length of a staged input row: N rounded up to RMAX modulo 32 words.
template <int R1, int R2> struct StageRow {
  static constexpr int N = R1 * R2 / 2, RM = Shape<R1, R2>::RMAX;
  static constexpr int NP = N + ((RM - N % 32) % 32 + 32) % 32;
};

// The inputs a launch group of pair fields reads, staged once per CTA by
// k_rows_fwd_multi: slot_of[i] is input i's staging slot (-1: unused).
struct RowsIn {
  int nin = 0;
  int8_t idx[kMaxIn] = {};
  int8_t slot_of[kMaxIn] = {};
};

// z forward for every field of a launch group: the L rows of each distinct
// input (the orbitals, psi) are staged in shared memory once, then each field's
// pair densities are formed straight into the stage-1 registers of its FFT.
// Same transform and output as k_rows_fwd, without re-reading the inputs per
// field. Stage-1 lanes read consecutive z of RMAX-lane lines, so a staged row
// is padded to a multiple of 32 words plus RMAX (StageRow): the lines a warp
// reads fall in disjoint bank ranges.
// BULK: one elected thread stages every row with a 1-D bulk copy
// (cp.async.bulk, one mbarrier for the whole block, a bounded wait), so the
// staging costs one round trip and no registers; used when every input is
// 16-byte aligned, a row and a padded staged row are multiples of 16 bytes
// and L divides the rows.
// Otherwise the threads stage with batches of 8 loads each.
template <typename T, int R1, int R2, int L, bool BULK>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_rows_fwd_multi(PassArgs args, RowsIn ri, int f0, int nfg, typename Cplx<T>::type* S1,
                     const typename Cplx<T>::type* tw, int* err) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, NP = StageRow<R1, R2>::NP, RM = Shape<R1, R2>::RMAX, NT = L * RM;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) uint64_t sbar;
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + L * RowBuf<R1, R2>::LS;
  T* stage = reinterpret_cast<T*>(tws + R1 * TwRow<T2, R2>::S);   // [slot][line][z], rows of NP
  const TwPrefetch<T2, R1 * TwRow<T2, R2>::S, NT> twp(tw);
  const int64_t row0 = (int64_t)blockIdx.x * L;
  const int64_t nrows = (int64_t)N * N;
  if constexpr (BULK) {
    __shared__ int s_misaligned;
    if (threadIdx.x == 0) {
      mbar_init(&sbar, 1);
      fence_barrier_init();
      // the host only picks this path for 16-byte aligned rows; re-check, and
      // record an error instead of issuing a copy that would fault
      int bad_align = (int)((smem_u32(stage) | (uint32_t)(NP * sizeof(T)) | (uint32_t)(N * sizeof(T))) & 15u);
      for (int sl = 0; sl < ri.nin; ++sl)
        bad_align |= (int)(reinterpret_cast<uintptr_t>(args.in[ri.idx[sl]]) & 15u);
      s_misaligned = bad_align;
      if (bad_align && err) atomicExch(err, 110);
    }
    __syncthreads();   // the barrier is initialised before anyone waits on it
    if (s_misaligned) return;
    if (threadIdx.x == 0) {
      mbar_expect_tx(&sbar, (uint32_t)(ri.nin * L * N * sizeof(T)));
      for (int sl = 0; sl < ri.nin; ++sl) {
        const T* src = reinterpret_cast<const T*>(args.in[ri.idx[sl]]) + row0 * N;
        for (int l = 0; l < L; ++l)
          bulk_load(stage + (sl * L + l) * NP, src + (int64_t)l * N, (uint32_t)(N * sizeof(T)), &sbar);
      }
    }
    twp.store(tws);
    bool bad = false;
    if (!mbar_wait_bounded(&sbar, 0, err, 108)) bad = true;
    if (__syncthreads_or(bad)) {
      if (threadIdx.x == 0) mbar_wait_bounded(&sbar, 0, err, 109);   // the copies still land
      return;
    }
  } else {
  // staging: 8 loads in flight per thread per batch (measured faster than one
  // batch of 32 at 128^3: 53 against 69 us)
  const int nel = ri.nin * L * N;
  constexpr int B = 8;
  for (int base = 0; base < nel; base += B * NT) {
    T v[B];
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const int i = base + threadIdx.x + k * NT;
      const int sl = i / (L * N), rem = i % (L * N);
      const int64_t r = row0 + rem / N;
      v[k] = (i < nel && r < nrows) ? reinterpret_cast<const T*>(args.in[ri.idx[sl]])[r * N + rem % N] : (T)0;
    }
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const int i = base + threadIdx.x + k * NT;
      if (i < nel) {
        const int sl = i / (L * N), rem = i % (L * N);
        stage[(sl * L + rem / N) * NP + rem % N] = v[k];
      }
    }
  }
  twp.store(tws);
  __syncthreads();
  }
  const int line = threadIdx.x / RM, j = threadIdx.x % RM;
  const int64_t r = row0 + line;
  for (int p = 0; p < nfg; ++p) {
    const FieldDesc& fd = args.f[f0 + p];
    if (j < R2) {
      const int a0 = ri.slot_of[fd.p[0].a];
      const int b0 = fd.p[0].b >= 0 ? ri.slot_of[fd.p[0].b] : -1;
      const int a1 = fd.p[1].a >= 0 ? ri.slot_of[fd.p[1].a] : -1;
      const int b1 = (a1 >= 0 && fd.p[1].b >= 0) ? ri.slot_of[fd.p[1].b] : -1;
      T2 v[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1 / 2; ++n1) {
        const int z = R2 * n1 + j;
        T x = stage[(a0 * L + line) * NP + z];
        if (b0 >= 0) x *= stage[(b0 * L + line) * NP + z];
        T y = (T)0;
        if (a1 >= 0) {
          y = stage[(a1 * L + line) * NP + z];
          if (b1 >= 0) y *= stage[(b1 * L + line) * NP + z];
        }
        v[n1].x = x;
        v[n1].y = y;
      }
      row_fwd_stage1<T2, R1, R2, true>(buf, line, j, v);
    }
    __syncthreads();
    if (j < R1) {
      T2 X[R2];
      row_fwd_stage2<T2, R1, R2>(buf, line, j, tws, X);
      if (r < nrows) {
        T2* d = S1 + (int64_t)p * nrows * M + r * M + j;
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) d[R1 * k2] = X[k2];
      }
    }
    __syncthreads();   // buf is rewritten by the next field
  }
}

// The bulk-staged z forward as a persistent kernel: each CTA walks row blocks
// blockIdx.x, blockIdx.x + gridDim.x, ... with the staging buffer doubled, so
// one elected thread issues the next block's row copies (1-D bulk copies on
// that buffer's mbarrier) before the current block is transformed and the
// copies land under the transforms. Same transforms and output as
// k_rows_fwd_multi. The host guarantees 16-byte aligned rows, a padded staged
// row that is a multiple of 16 bytes and L | N^2; the kernel re-checks the
// alignment and records error 110 instead of issuing a bad copy. Waits are
// bounded (codes 113/114).
template <typename T, int R1, int R2, int L>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_rows_fwd_pers(PassArgs args, RowsIn ri, int f0, int nfg, typename Cplx<T>::type* S1,
                    const typename Cplx<T>::type* tw, int* err) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, NP = StageRow<R1, R2>::NP, RM = Shape<R1, R2>::RMAX, NT = L * RM;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) uint64_t sbar[2];
  __shared__ int s_misaligned;
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + L * RowBuf<R1, R2>::LS;
  T* stage0 = reinterpret_cast<T*>(tws + R1 * TwRow<T2, R2>::S);   // [slot][input][line][z], rows of NP
  const int SB = ri.nin * L * NP;                                    // floats per staging slot
  const int64_t nrows = (int64_t)N * N;
  const int nblk = (int)(nrows / L);
  if (threadIdx.x == 0) {
    mbar_init(&sbar[0], 1);
    mbar_init(&sbar[1], 1);
    fence_barrier_init();
    int bad_align = (int)((smem_u32(stage0) | (uint32_t)(SB * sizeof(T)) | (uint32_t)(NP * sizeof(T)) |
                           (uint32_t)(N * sizeof(T))) & 15u);
    for (int sl = 0; sl < ri.nin; ++sl)
      bad_align |= (int)(reinterpret_cast<uintptr_t>(args.in[ri.idx[sl]]) & 15u);
    s_misaligned = bad_align;
    if (bad_align && err) atomicExch(err, 110);
  }
  for (int i = threadIdx.x; i < R1 * TwRow<T2, R2>::S; i += NT) tws[i] = tw[i];
  __syncthreads();
  if (s_misaligned) return;
  auto issue = [&](int blk, int slot) {
    mbar_expect_tx(&sbar[slot], (uint32_t)(ri.nin * L * N * sizeof(T)));
    T* st = stage0 + slot * SB;
    for (int sl = 0; sl < ri.nin; ++sl) {
      const T* src = reinterpret_cast<const T*>(args.in[ri.idx[sl]]) + (int64_t)blk * L * N;
      for (int l = 0; l < L; ++l)
        bulk_load(st + (sl * L + l) * NP, src + (int64_t)l * N, (uint32_t)(N * sizeof(T)), &sbar[slot]);
    }
  };
  if (threadIdx.x == 0 && (int)blockIdx.x < nblk) issue(blockIdx.x, 0);
  const int line = threadIdx.x / RM, j = threadIdx.x % RM;
  int it = 0;
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x, ++it) {
    const int slot = it & 1;
    // the other slot was last read by the previous block, which ended at a barrier
    const bool more = blk + (int)gridDim.x < nblk;
    if (threadIdx.x == 0 && more) issue(blk + gridDim.x, slot ^ 1);
    const bool bad = !mbar_wait_bounded(&sbar[slot], (it >> 1) & 1, err, 113);
    if (__syncthreads_or(bad)) {
      if (threadIdx.x == 0) {   // copies still in flight land before the CTA goes away
        mbar_wait_bounded(&sbar[slot], (it >> 1) & 1, err, 114);
        if (more) mbar_wait_bounded(&sbar[slot ^ 1], ((it + 1) >> 1) & 1, err, 114);
      }
      return;
    }
    const T* stage = stage0 + slot * SB;
    const int64_t r = (int64_t)blk * L + line;
    for (int p = 0; p < nfg; ++p) {
      const FieldDesc& fd = args.f[f0 + p];
      if (j < R2) {
        const int a0 = ri.slot_of[fd.p[0].a];
        const int b0 = fd.p[0].b >= 0 ? ri.slot_of[fd.p[0].b] : -1;
        const int a1 = fd.p[1].a >= 0 ? ri.slot_of[fd.p[1].a] : -1;
        const int b1 = (a1 >= 0 && fd.p[1].b >= 0) ? ri.slot_of[fd.p[1].b] : -1;
        T2 v[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1 / 2; ++n1) {
          const int z = R2 * n1 + j;
          T x = stage[(a0 * L + line) * NP + z];
          if (b0 >= 0) x *= stage[(b0 * L + line) * NP + z];
          T y = (T)0;
          if (a1 >= 0) {
            y = stage[(a1 * L + line) * NP + z];
            if (b1 >= 0) y *= stage[(b1 * L + line) * NP + z];
          }
          v[n1].x = x;
          v[n1].y = y;
        }
        row_fwd_stage1<T2, R1, R2, true>(buf, line, j, v);
      }
      fence_proxy_async_smem();   // this slot's reads precede the copies issued into it next
      __syncthreads();
      if (j < R1) {
        T2 X[R2];
        row_fwd_stage2<T2, R1, R2>(buf, line, j, tws, X);
        T2* d = S1 + (int64_t)p * nrows * M + r * M + j;
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) d[R1 * k2] = X[k2];
      }
      __syncthreads();   // buf is rewritten by the next field; the stage slot is free after the last
    }
  }
}

// z inverse over every field of the group, then the epilogue. NO > 0: the
// accumulation terms target outputs < NO, kept in registers (each thread owns
// the R1/2 fixed elements z = j + R2 n1 of its row); NO == 0: energy mode.
// FP32, one output, M = 256 fits 64 registers without spills: four CTAs per SM.
template <typename T, int R1, int R2, int NO>
constexpr int rows_inv_min_ctas() {
  return (NO == 1 && sizeof(T) == 4 && R1 == 16 && R2 == 16) ? 4 : 1;
}

template <typename T, int R1, int R2, int L, int NO>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX, (rows_inv_min_ctas<T, R1, R2, NO>()))
    k_rows_inv(PassArgs args, int f0, int nfg, const typename Cplx<T>::type* S1,
               const typename Cplx<T>::type* tw, int accumulate, double* partials,
               int64_t slot_stride) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, RM = Shape<R1, R2>::RMAX, NT = L * RM;
  constexpr int EPT = R1 / 2;
  constexpr bool ENERGY = NO == 0;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sh[32];
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + L * RowBuf<R1, R2>::LS;
  const TwPrefetch<T2, R1 * TwRow<T2, R2>::S, NT> twp(tw);
  const int64_t nrows = (int64_t)N * N;
  const int line = threadIdx.x / RM, j = threadIdx.x % RM;
  const int64_t r = (int64_t)blockIdx.x * L + line;
  const bool own = j < R2 && r < nrows;   // this thread owns elements of the output
  T acc[ENERGY ? 1 : NO][EPT];
#pragma unroll
  for (int o = 0; o < (ENERGY ? 1 : NO); ++o)
#pragma unroll
    for (int e = 0; e < EPT; ++e) acc[o][e] = (T)0;
  Acc<T> e0, e1;
  for (int p = 0; p < nfg; ++p) {
    const FieldDesc& fd = args.f[f0 + p];
    // The epilogue's first field factor of each part (in[tc] of term 0, or the
    // density in energy mode) does not depend on the transform. With several
    // outputs (or energies) it is loaded now, so its latency overlaps the FFT;
    // with one output it is loaded in the epilogue, which keeps the kernel at
    // four CTAs per SM (64 registers). A second term (block applies on the
    // generic engine only) always loads in the epilogue.
    constexpr bool PREFETCH = ENERGY || NO > 1;
    T fac[EPT][2];
    auto load_fac = [&]() {
#pragma unroll
      for (int e = 0; e < EPT; ++e) {
        const int64_t gi = r * N + j + R2 * e;
#pragma unroll
        for (int qq = 0; qq < 2; ++qq) {
          const PartDesc& d = fd.p[qq];
          if constexpr (ENERGY)
            fac[e][qq] = (own && d.a >= 0) ? dens<T>(d, args.in, gi) : (T)0;
          else
            fac[e][qq] = (own && d.a >= 0 && d.nt > 0)
                             ? (d.tc[0] >= 0 ? reinterpret_cast<const T*>(args.in[d.tc[0]])[gi] : (T)1)
                             : (T)0;
        }
      }
    };
    if constexpr (PREFETCH) load_fac();
    T2 X[R2];
    if (j < R1) {
      const T2* src = S1 + (int64_t)p * nrows * M + r * M + j;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        if (r < nrows) X[k2] = src[R1 * k2];
        else X[k2].x = X[k2].y = 0;
      }
    }
    if (p == 0) twp.store(tws);
    __syncthreads();   // tws is visible; the previous field's stage-B reads of buf are done
    if (j < R1) row_inv_stageA<T2, R1, R2>(buf, line, j, tws, X);
    __syncthreads();
    if (own) {
      if constexpr (!PREFETCH) load_fac();
      T2 w[R1];
      row_inv_stageB<T2, R1, R2>(buf, line, j, w);
#pragma unroll
      for (int e = 0; e < EPT; ++e) {
        const int64_t gi = r * N + j + R2 * e;
        const T2 J = w[e];
#pragma unroll
        for (int qq = 0; qq < 2; ++qq) {
          const PartDesc& d = fd.p[qq];
          if (d.a < 0) continue;
          const T val = qq == 0 ? J.x : J.y;
          if constexpr (ENERGY) {
            const T de = fac[e][qq];
            if (d.eslot == 0) e0.add_prod(de * (T)d.ew, val);
            else e1.add_prod(de * (T)d.ew, val);
          } else {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              if (k >= d.nt) break;
              T m = (T)d.coef[k];
              if (k == 0) m *= fac[e][qq];
              else if (d.tc[1] >= 0) m *= reinterpret_cast<const T*>(args.in[d.tc[1]])[gi];
              const int to = d.to[k];
#pragma unroll
              for (int o = 0; o < NO; ++o)
                if (o == to) acc[o][e] += m * val;
            }
          }
        }
      }
    }
  }
  if constexpr (ENERGY) {
    const double s0 = block_sum(e0.value(), sh);
    const double s1 = block_sum(e1.value(), sh);
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = s0;
      partials[slot_stride + blockIdx.x] = s1;
    }
  } else {
    if (!own) return;
    const int nout = args.nout;
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      if (o >= nout) break;
      T* dst = reinterpret_cast<T*>(args.out[o]) + r * N + j;
#pragma unroll
      for (int e = 0; e < EPT; ++e) dst[R2 * e] = accumulate ? dst[R2 * e] + acc[o][e] : acc[o][e];
    }
  }
}

// z inverse of one field per CTA (grid.y = field), writing J_re and J_im of
// the row block to their own real fields (the EPI_J epilogue).
template <typename T, int R1, int R2, int L>
__global__ void __launch_bounds__(L * Shape<R1, R2>::RMAX)
    k_rows_inv_j(T* jbase, int64_t jstride, int f0, const typename Cplx<T>::type* S1,
                 const typename Cplx<T>::type* tw) {
  using T2 = typename Cplx<T>::type;
  constexpr int M = R1 * R2, N = M / 2, RM = Shape<R1, R2>::RMAX, NT = L * RM;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* buf = reinterpret_cast<T2*>(smraw);
  T2* tws = buf + L * RowBuf<R1, R2>::LS;
  const TwPrefetch<T2, R1 * TwRow<T2, R2>::S, NT> twp(tw);
  const int p = blockIdx.y;
  const int64_t nrows = (int64_t)N * N;
  const int line = threadIdx.x / RM, j = threadIdx.x % RM;
  const int64_t r = (int64_t)blockIdx.x * L + line;
  T2 X[R2];
  if (j < R1) {
    const T2* src = S1 + (int64_t)p * nrows * M + r * M + j;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) {
      if (r < nrows) X[k2] = src[R1 * k2];
      else X[k2].x = X[k2].y = 0;
    }
  }
  twp.store(tws);
  __syncthreads();
  if (j < R1) row_inv_stageA<T2, R1, R2>(buf, line, j, tws, X);
  __syncthreads();
  if (j < R2 && r < nrows) {
    T2 w[R1];
    row_inv_stageB<T2, R1, R2>(buf, line, j, w);
    T* jre = jbase + (int64_t)(2 * (f0 + p)) * jstride + r * N + j;
    T* jim = jre + jstride;
#pragma unroll
    for (int n1 = 0; n1 < R1 / 2; ++n1) {
      jre[R2 * n1] = w[n1].x;
      jim[R2 * n1] = w[n1].y;
    }
  }
}

template <typename K>
inline int smem_attr(K k, size_t bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(k), bytes);
}

// Launchers for one shape.
template <typename T, int R1, int R2, int L>
struct Launch {
  using T2 = typename Cplx<T>::type;
  static constexpr int M = R1 * R2, N = M / 2, NT = L * Shape<R1, R2>::RMAX;
  static constexpr int TWN = R1 * TwRow<T2, R2>::S;   // stage-twiddle table entries
  static size_t sm_cols() { return (size_t)(M * (L + 1) + TWN) * sizeof(T2); }
  static size_t sm_rows() { return (size_t)(L * RowBuf<R1, R2>::LS + TWN) * sizeof(T2); }
  static int cols(int mode, const T2* in, T2* out, const ColGeom& g, int outer, int nf, const T2* tw,
                  const T* ghat, int H, cudaStream_t s) {
    if (g.ncols % L == 0) return cols_t<true>(mode, in, out, g, outer, nf, tw, ghat, H, s);
    return cols_t<false>(mode, in, out, g, outer, nf, tw, ghat, H, s);
  }
  template <bool FULL>
  static int cols_t(int mode, const T2* in, T2* out, const ColGeom& g, int outer, int nf, const T2* tw,
                    const T* ghat, int H, cudaStream_t s) {
    dim3 grid(outer, (g.ncols + L - 1) / L, nf);
    const size_t sm = sm_cols();
    if (mode == COL_FWD) {
      GATO_TRY(smem_attr(k_cols<T, R1, R2, L, COL_FWD, FULL>, sm));
      k_cols<T, R1, R2, L, COL_FWD, FULL><<<grid, NT, sm, s>>>(in, out, g, tw, ghat, H);
    } else if (mode == COL_INV) {
      GATO_TRY(smem_attr(k_cols<T, R1, R2, L, COL_INV, FULL>, sm));
      k_cols<T, R1, R2, L, COL_INV, FULL><<<grid, NT, sm, s>>>(in, out, g, tw, ghat, H);
    } else {
      GATO_TRY(smem_attr(k_cols<T, R1, R2, L, COL_FMI, FULL>, sm));
      k_cols<T, R1, R2, L, COL_FMI, FULL><<<grid, NT, sm, s>>>(in, out, g, tw, ghat, H);
    }
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  static int cols_fe(const T2* in, const ColGeom& g, int outer, int nf, const T2* tw, const T* ghat, int H,
                     const FeArgs& fa, cudaStream_t s) {
    dim3 grid(outer, (g.ncols + L - 1) / L, nf);
    const size_t sm = sm_cols();
    if (g.ncols % L == 0) {
      GATO_TRY(smem_attr(k_cols_fe<T, R1, R2, L, true>, sm));
      k_cols_fe<T, R1, R2, L, true><<<grid, NT, sm, s>>>(in, g, tw, ghat, H, fa);
    } else {
      GATO_TRY(smem_attr(k_cols_fe<T, R1, R2, L, false>, sm));
      k_cols_fe<T, R1, R2, L, false><<<grid, NT, sm, s>>>(in, g, tw, ghat, H, fa);
    }
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  // multi: 0 per-field CTAs, 1 multi-field CTAs from three fields up, 2 from two fields up
  // (persistent, double-buffered staging where the rows allow bulk copies), 3 as 2 with one
  // staging round trip per CTA (the non-persistent kernel)
  // (the default: with bulk staging the multi-field kernel wins at two fields too,
  // 239 against 244 us for the 128^3 matvec)
  static int rows_fwd(const PassArgs& a, int f0, int nfg, T2* S1, const T2* tw, int multi, cudaStream_t s) {
    // several fields over few distinct inputs: stage the inputs once per CTA
    RowsIn ri;
    for (int i = 0; i < kMaxIn; ++i) ri.slot_of[i] = -1;
    auto use = [&](int idx) {
      if (idx < 0 || ri.slot_of[idx] >= 0) return;
      ri.slot_of[idx] = (int8_t)ri.nin;
      ri.idx[ri.nin++] = (int8_t)idx;
    };
    for (int p = 0; p < nfg; ++p)
      for (int qq = 0; qq < 2; ++qq) {
        const PartDesc& d = a.f[f0 + p].p[qq];
        if (d.a < 0) continue;
        use(d.a);
        use(d.b);
      }
    // half the rows per CTA of the other z kernels: the grid covers every
    // field at once, so smaller CTAs give more of them and a shorter last wave
    constexpr int LM = L >= 16 ? L / 2 : L;
    const size_t stage_bytes = (size_t)ri.nin * LM * StageRow<R1, R2>::NP * sizeof(T);
    if (multi > 0 && nfg >= (multi == 1 ? 3 : 2) && stage_bytes <= 48 * 1024) {
      const size_t sm = (size_t)(LM * RowBuf<R1, R2>::LS + TWN) * sizeof(T2) + stage_bytes;
      const int64_t nrows = (int64_t)N * N;
      // a bulk copy needs 16-byte aligned source and destination rows and a
      // size that is a multiple of 16 bytes (the padded staged row included)
      bool bulk = nrows % LM == 0 && (N * sizeof(T)) % 16 == 0 &&
                  (StageRow<R1, R2>::NP * sizeof(T)) % 16 == 0;
      for (int i = 0; i < ri.nin; ++i) bulk = bulk && ((uintptr_t)a.in[ri.idx[i]] % 16) == 0;
      const unsigned grid = (unsigned)((nrows + LM - 1) / LM);
      if (bulk && multi != 3) {
        // persistent CTAs over the row blocks, double-buffered staging: one resident wave
        auto kern = k_rows_fwd_pers<T, R1, R2, LM>;
        const size_t smp = sm + stage_bytes;   // a second staging slot
        GATO_TRY(smem_attr(kern, smp));
        static std::atomic<int> wave[kMaxIn + 1];   // resident blocks of one wave by staged inputs (0: unknown)
        int w = wave[ri.nin].load();
        if (w == 0) {
          int dev = 0, sms = 0, ps = 0;
          GATO_CUDA_TRY(cudaGetDevice(&dev));
          GATO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
          GATO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, kern, LM * Shape<R1, R2>::RMAX, smp));
          if (ps < 1) return fail(GATO_EUNSUPPORTED, "z forward: no resident CTA fits");
          w = ps * sms;
          wave[ri.nin].store(w);
        }
        const unsigned pg = (unsigned)std::min<int64_t>(grid, (int64_t)w);
        kern<<<pg, LM * Shape<R1, R2>::RMAX, smp, s>>>(a, ri, f0, nfg, S1, tw, device_error_word());
      } else if (bulk) {
        GATO_TRY(smem_attr(k_rows_fwd_multi<T, R1, R2, LM, true>, sm));
        k_rows_fwd_multi<T, R1, R2, LM, true><<<grid, LM * Shape<R1, R2>::RMAX, sm, s>>>(
            a, ri, f0, nfg, S1, tw, device_error_word());
      } else {
        GATO_TRY(smem_attr(k_rows_fwd_multi<T, R1, R2, LM, false>, sm));
        k_rows_fwd_multi<T, R1, R2, LM, false><<<grid, LM * Shape<R1, R2>::RMAX, sm, s>>>(
            a, ri, f0, nfg, S1, tw, device_error_word());
      }
      GATO_LAUNCH_TRY();
      return GATO_OK;
    }
    const size_t sm = sm_rows();
    GATO_TRY(smem_attr(k_rows_fwd<T, R1, R2, L>, sm));
    const int64_t nrows = (int64_t)N * N;
    k_rows_fwd<T, R1, R2, L><<<dim3((unsigned)((nrows + L - 1) / L), nfg), NT, sm, s>>>(a, f0, S1, tw);
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  template <int NO>
  static int rows_inv_no(const PassArgs& a, int f0, int nfg, const T2* S1, const T2* tw, int accumulate,
                         double* partials, int64_t slot_stride, cudaStream_t s) {
    const size_t sm = sm_rows();
    const unsigned nblk = (unsigned)(((int64_t)N * N + L - 1) / L);
    GATO_TRY(smem_attr(k_rows_inv<T, R1, R2, L, NO>, sm));
    k_rows_inv<T, R1, R2, L, NO><<<nblk, NT, sm, s>>>(a, f0, nfg, S1, tw, accumulate, partials,
                                                       slot_stride);
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  static int rows_inv_j(const PassArgs& a, int f0, int nfg, const T2* S1, const T2* tw, cudaStream_t s) {
    const size_t sm = sm_rows();
    const unsigned nblk = (unsigned)(((int64_t)N * N + L - 1) / L);
    GATO_TRY(smem_attr(k_rows_inv_j<T, R1, R2, L>, sm));
    k_rows_inv_j<T, R1, R2, L><<<dim3(nblk, nfg), NT, sm, s>>>((T*)a.jbase, a.jstride, f0, S1, tw);
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  static int rows_inv(const PassArgs& a, int f0, int nfg, const T2* S1, const T2* tw, int accumulate,
                      bool energy, double* partials, int64_t slot_stride, cudaStream_t s) {
    if (energy) return rows_inv_no<0>(a, f0, nfg, S1, tw, accumulate, partials, slot_stride, s);
    if (a.nout <= 1) return rows_inv_no<1>(a, f0, nfg, S1, tw, accumulate, partials, slot_stride, s);
    if (a.nout <= 2) return rows_inv_no<2>(a, f0, nfg, S1, tw, accumulate, partials, slot_stride, s);
    if (a.nout <= 4) return rows_inv_no<4>(a, f0, nfg, S1, tw, accumulate, partials, slot_stride, s);
    return rows_inv_no<8>(a, f0, nfg, S1, tw, accumulate, partials, slot_stride, s);
  }
};

}  // namespace fast
}  // namespace gato
