// Finite-difference Laplacian / Hamiltonian apply (operators.py:40-130,
// hamiltonian.py:25-31).
//
// Hot path (Dirichlet, 16-byte aligned rows): each CTA owns a 32 (y) x 32 (z)
// column of the grid and marches along x through a chunk of planes. One
// elected thread streams (32+2R) x (32+2A) halo planes into a 6-slot
// shared-memory ring with TMA (cp.async.bulk.tensor, mbarrier completion);
// the tensor map's zero out-of-bounds fill is exactly the reference's zero
// padding, so no boundary branches exist. Each thread owns a z pair of 4 (or
// 2) rows: x-neighbours live in a per-thread register queue, y/z neighbours
// are pair reads of the centre plane in shared memory. The 32 x 32 V tile of
// each centre plane rides in the same ring slot (a second tensor map, same
// mbarrier), so V arrives with the ring's look-ahead instead of one DRAM
// round trip per plane; the output is a coalesced pair store. HBM-bound: the
// algorithmic traffic is 3 N^3 s bytes (psi, V, out).
#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <type_traits>
#include <utility>

#include "common.cuh"
#include "ptx.cuh"
#include "stencil.cuh"

namespace gato {

namespace {

template <typename T>
struct StencilCoef {
  T c0, c1, c2;
};

template <typename T>
__host__ __device__ inline StencilCoef<T> coefs(int order) {
  if (order == 2) return {(T)-6.0, (T)1.0, (T)0.0};
  return {(T)(3.0 * (-30.0 / 12.0)), (T)(16.0 / 12.0), (T)(-1.0 / 12.0)};
}

// Laplacian sum from the centre value and the neighbour sums. The FP32 path
// uses differences to the centre (sum_k c_k (psi_k - psi_0)), which removes
// the cancellation of the c0 term; FP64 keeps the direct form, cheaper on
// GB300's narrow FP64 pipe.
template <typename T>
__device__ __forceinline__ T lap_combine(T ctr, T s1, T s2, StencilCoef<T> c, int R) {
  if constexpr (sizeof(T) == 4) {
    T d1 = s1 - (T)6 * ctr;
    T d2 = (R == 2) ? (s2 - (T)6 * ctr) : (T)0;
    return c.c1 * d1 + c.c2 * d2;
  } else {
    return c.c0 * ctr + c.c1 * s1 + c.c2 * s2;
  }
}

// ---- generic kernel: any shape, both boundaries -----------------------------------
template <typename T, int R, bool PERIODIC>
__global__ void k_stencil_generic(const T* __restrict__ psi, const T* __restrict__ V,
                                  T* __restrict__ out, int nb, int nx, int ny, int nz,
                                  int64_t bstride, T coef, double* dot_part) {
  __shared__ double sh[32];
  StencilCoef<T> c = coefs<T>(R == 1 ? 2 : 4);
  int64_t n3 = (int64_t)nx * ny * nz;
  int64_t total = n3 * nb;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // dot partials are per batch: require the grid to cover one batch per
  // blockIdx.y when dot_part is requested.
  int b_lo = dot_part ? blockIdx.y : 0;
  int b_hi = dot_part ? blockIdx.y + 1 : nb;
  Acc<T> acc;
  for (int b = b_lo; b < b_hi; ++b) {
    const T* p = psi + (int64_t)b * bstride;
    T* o = out + (int64_t)b * bstride;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += stride) {
      int z = (int)(i % nz);
      int64_t t = i / nz;
      int y = (int)(t % ny);
      int x = (int)(t / ny);
      auto at = [&](int xx, int yy, int zz) -> T {
        if (PERIODIC) {
          xx = (xx % nx + nx) % nx;
          yy = (yy % ny + ny) % ny;
          zz = (zz % nz + nz) % nz;
        } else if (xx < 0 || xx >= nx || yy < 0 || yy >= ny || zz < 0 || zz >= nz) {
          return (T)0;
        }
        return p[((int64_t)xx * ny + yy) * nz + zz];
      };
      T ctr = p[i];
      T s1 = at(x - 1, y, z) + at(x + 1, y, z) + at(x, y - 1, z) + at(x, y + 1, z) +
             at(x, y, z - 1) + at(x, y, z + 1);
      T s2 = (T)0;
      if (R == 2)
        s2 = at(x - 2, y, z) + at(x + 2, y, z) + at(x, y - 2, z) + at(x, y + 2, z) +
             at(x, y, z - 2) + at(x, y, z + 2);
      T val = coef * lap_combine<T>(ctr, s1, s2, c, R);
      if (V) val += V[i] * ctr;
      if (out) o[i] = val;
      if (dot_part) acc.add_prod(ctr, val);
    }
  }
  (void)total;
  if (dot_part) {
    double v = block_sum(acc.value(), sh);
    if (threadIdx.x == 0) dot_part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = v;
  }
}

// ---- TMA plane-marching kernel ---------------------------------------------------
constexpr int kBZ = 32;       // tile width along z
constexpr int kBY = 32;       // tile height along y
constexpr int kZP = kBZ / 2;  // threads along z: each owns two consecutive z points
constexpr int kSlots = 6;     // plane ring depth: 3 planes of look-ahead, 3 FP32 (2 FP64) CTAs per SM

template <typename T> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };

template <typename T>
__device__ __forceinline__ typename Pair<T>::type ld2(const T* p) {
  return *reinterpret_cast<const typename Pair<T>::type*>(p);
}

template <typename T, int R>
struct TmaGeom {
  static constexpr int A = 16 / (int)sizeof(T);  // z halo, rounded to 16 bytes
  static constexpr int PW = kBZ + 2 * A;
  static constexpr int PH = kBY + 2 * R;
  static constexpr int BOX_BYTES = PW * PH * (int)sizeof(T);
  static constexpr int V_OFF = (BOX_BYTES + 127) / 128 * 128;   // V tile inside the slot
  static constexpr int V_BYTES = kBZ * kBY * (int)sizeof(T);
  static constexpr int SLOT_BYTES = V_OFF + (V_BYTES + 127) / 128 * 128;
  static constexpr int SMEM = kSlots * SLOT_BYTES + kSlots * 8 + 128;
};

// Runs step(slot 0), step(slot 1), ... in order until one returns false.
template <typename F, int... Js>
__device__ __forceinline__ bool run_slots(F& step, int qb, std::integer_sequence<int, Js...>) {
  return (step(std::integral_constant<int, Js>{}, qb) && ...);
}

// One CTA: a kBY x kBZ column of one field, planes [xs, xs + cx) along x.
// Plane q of the chunk is x = xs - R + q and sits in ring slot q % kSlots; it
// feeds the x register queue at iteration q and is the centre plane at
// iteration q + R, after which its slot is refilled with plane q + kSlots.
// The plane loop is unrolled by the ring depth, so slot addresses are
// immediates and the queue shifts are register renames. Each thread owns the
// z pair (z, z + 1) of YPT consecutive rows: every shared-memory access moves
// a pair (8 bytes FP32, 16 bytes FP64), the z neighbours of both points come
// from two pair loads (z - 2, z - 1) and (z + 2, z + 3), the y neighbours are
// the thread's own queue centres plus 2R halo rows, and the output leaves as
// one pair store per row.
template <typename T, int R, int YPT, bool HAS_V, bool STORE, bool DOT>
__global__ void __launch_bounds__(kZP*(kBY / YPT))
    k_stencil_tma(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap vmap,
                  T* __restrict__ out, int nx, int ny, int nz, int cx, int tiles_z, int64_t bstride,
                  T coef, double* dot_part, int* err) {
  using G = TmaGeom<T, R>;
  using P2 = typename Pair<T>::type;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 128-byte aligned ring; offsetting the shared array itself keeps every
  // ring access a shared-memory access
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kSlots * G::SLOT_BYTES);
  __shared__ double sh[32];

  const StencilCoef<T> c = coefs<T>(R == 1 ? 2 : 4);
  const int tz = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * kZP + tz;
  const int tile_z = blockIdx.x % tiles_z, tile_y = blockIdx.x / tiles_z;
  const int z0 = tile_z * kBZ, y0 = tile_y * kBY;
  const int xs = blockIdx.y * cx;
  const int xe = min(xs + cx, nx);
  const int P = xe - xs + 2 * R;
  const int b = blockIdx.z;

  if (tid == 0) {
    for (int s = 0; s < kSlots; ++s) mbar_init(&bars[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  // Only the centre planes R <= q < P - R carry a V tile.
  auto issue = [&](int q) {
    const int s = q % kSlots;
    const bool v = HAS_V && q >= R && q < P - R;
    mbar_expect_tx(&bars[s], G::BOX_BYTES + (v ? G::V_BYTES : 0));
    tma_load_4d(smem + s * G::SLOT_BYTES, &tmap, &bars[s], z0 - G::A, y0 - R, xs - R + q, b);
    if (v) tma_load_3d(smem + s * G::SLOT_BYTES + G::V_OFF, &vmap, &bars[s], z0, y0, xs - R + q);
  };
  int issued = 0;   // meaningful in thread 0 only
  if (tid == 0) {
    issued = P < kSlots ? P : kSlots;
    for (int q = 0; q < issued; ++q) issue(q);
  }

  const int yt = ty * YPT;
  const int gz = z0 + 2 * tz;   // nz is even, so a pair is wholly inside or outside
  unsigned live = 0;
#pragma unroll
  for (int k = 0; k < YPT; ++k)
    if (gz < nz && y0 + yt + k < ny) live |= 1u << k;
  T* obase = nullptr;
  if (STORE) obase = out + (int64_t)b * bstride + ((int64_t)xs * ny + (y0 + yt)) * nz + gz;
  const int64_t pstride = (int64_t)ny * nz;
  const int cidx = (yt + R) * G::PW + 2 * tz + G::A;   // first row, centre pair (even index)
  const int vidx = yt * kBZ + 2 * tz;

  P2 xq[YPT][2 * R + 1];
#pragma unroll
  for (int k = 0; k < YPT; ++k)
#pragma unroll
    for (int r = 0; r < 2 * R + 1; ++r) xq[k][r].x = xq[k][r].y = (T)0;
  Acc<T> acc;
  bool bad = false;
  int q = 0;
  T* op = obase;   // output row of the next centre plane
  // One plane step with ring slot J a compile-time constant, so slot addresses
  // are immediates and the x-queue shifts are register renames; false ends
  // the march (end of the chunk, or a timed-out wait anywhere in the CTA).
  auto step = [&](auto slot, int qb) -> bool {
    constexpr int J = decltype(slot)::value;
    q = qb + J;
    if (q >= P) return false;
    if (!mbar_wait_bounded(&bars[J], (uint32_t)((qb / kSlots) & 1), err, 101)) bad = true;
    const T* pl = reinterpret_cast<const T*>(smem + J * G::SLOT_BYTES);
#pragma unroll
    for (int k = 0; k < YPT; ++k) {
#pragma unroll
      for (int r = 0; r < 2 * R; ++r) xq[k][r] = xq[k][r + 1];
      xq[k][2 * R] = ld2(pl + cidx + k * G::PW);
    }
    if (q >= 2 * R) {
      constexpr int CS = (J + kSlots - R) % kSlots;
      const T* pc = reinterpret_cast<const T*>(smem + CS * G::SLOT_BYTES);
      [[maybe_unused]] const T* pv = reinterpret_cast<const T*>(smem + CS * G::SLOT_BYTES + G::V_OFF);
      P2 col[YPT + 2 * R];
#pragma unroll
      for (int i = 0; i < R; ++i) {
        col[i] = ld2(pc + cidx + (i - R) * G::PW);
        col[R + YPT + i] = ld2(pc + cidx + (YPT + i) * G::PW);
      }
#pragma unroll
      for (int k = 0; k < YPT; ++k) col[R + k] = xq[k][R];
#pragma unroll
      for (int k = 0; k < YPT; ++k) {
        const int idx = cidx + k * G::PW;
        const P2 ctr = xq[k][R];
        const P2 lo = ld2(pc + idx - 2), hi = ld2(pc + idx + 2);   // (z-2, z-1), (z+2, z+3)
        // point z in .x, point z + 1 in .y; neighbour order x, y, z as in the reference sum
        T s1a = xq[k][R - 1].x + xq[k][R + 1].x + col[R + k - 1].x + col[R + k + 1].x + lo.y + ctr.y;
        T s1b = xq[k][R - 1].y + xq[k][R + 1].y + col[R + k - 1].y + col[R + k + 1].y + ctr.x + hi.x;
        T s2a = (T)0, s2b = (T)0;
        if constexpr (R == 2) {
          s2a = xq[k][0].x + xq[k][4].x + col[k].x + col[k + 4].x + lo.x + hi.x;
          s2b = xq[k][0].y + xq[k][4].y + col[k].y + col[k + 4].y + lo.y + hi.y;
        }
        P2 val;
        val.x = coef * lap_combine<T>(ctr.x, s1a, s2a, c, R);
        val.y = coef * lap_combine<T>(ctr.y, s1b, s2b, c, R);
        if constexpr (HAS_V) {
          const P2 v = ld2(pv + vidx + k * kBZ);
          val.x += v.x * ctr.x;
          val.y += v.y * ctr.y;
        }
        if (live & (1u << k)) {
          if constexpr (STORE) *reinterpret_cast<P2*>(op + k * nz) = val;
          if constexpr (DOT) {
            acc.add_prod(ctr.x, val.x);
            acc.add_prod(ctr.y, val.y);
          }
        }
      }
      if constexpr (STORE) op += pstride;
    }
    // every thread is done with plane q - R; a timed-out wait anywhere stops the CTA
    fence_proxy_async_smem();   // its slot's reads precede the copy issued into it below
    if (__syncthreads_or(bad)) {
      bad = true;
      return false;
    }
    if (tid == 0 && q >= R && q - R + kSlots < P) {
      issue(q - R + kSlots);
      ++issued;
    }
    return true;
  };
  for (int qb = 0; qb < P; qb += kSlots)
    if (!run_slots(step, qb, std::make_integer_sequence<int, kSlots>{})) break;
  if (bad) {
    // drain the copies still in flight (bounded) before the CTA's shared memory goes away
    if (tid == 0)
      for (int p = q; p < issued; ++p)
        mbar_wait_bounded(&bars[p % kSlots], (uint32_t)((p / kSlots) & 1), err, 102);
    return;
  }
  if constexpr (DOT) {
    double v = block_sum(acc.value(), sh);
    if (tid == 0)
      dot_part[(int64_t)b * gridDim.x * gridDim.y + (int64_t)blockIdx.y * gridDim.x + blockIdx.x] =
          v;
  }
}

// Rows per thread of the TMA kernel: 4 (128-thread CTAs) or 2 (256-thread
// CTAs); 0 picks the default. Process-wide, set by the autotuner.
std::atomic<int> g_rows_per_thread{0};
constexpr int kDefaultRows = 2;

// Resident CTAs of a kernel on the whole GPU (occupancy x SMs).
template <typename K>
int resident_ctas(K kernel, int threads, int smem) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess ||
      per <= 0)
    return 152;
  return per * sms;
}

template <typename T, int R, int YPT, bool HAS_V, bool STORE, bool DOT>
int launch_tma_rows(const CUtensorMap& tm, const CUtensorMap& vm, void* out, int nb, int nx, int ny,
                    int nz, int64_t bstride, double coef, double* dot_part, int* nparts,
                    cudaStream_t s) {
  using G = TmaGeom<T, R>;
  constexpr int kThreads = kZP * (kBY / YPT);
  auto kern = k_stencil_tma<T, R, YPT, HAS_V, STORE, DOT>;
  // opt in to the large shared-memory carve-out once per device (the launch
  // itself then issues only stream work, so it can be graph-captured)
  static std::atomic<unsigned> attr_done{0};
  int dev = 0;
  GATO_CUDA_TRY(cudaGetDevice(&dev));
  const unsigned bit = 1u << (dev & 31);
  if (!(attr_done.load() & bit)) {
    GATO_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM));
    attr_done.fetch_or(bit);
  }
  const int tiles_z = (nz + kBZ - 1) / kBZ, tiles_y = (ny + kBY - 1) / kBY;
  const int tiles = tiles_z * tiles_y;
  // Split x into chunks so the grid is one full resident wave where the
  // problem allows (every CTA streams at once, no tail wave); a chunk keeps at
  // least 4 planes, since its 2R halo planes are re-read.
  static const int cap = resident_ctas(kern, kThreads, G::SMEM);   // one value per instantiation
  int chunks = (int)std::max<int64_t>(1, cap / ((int64_t)tiles * nb));
  chunks = std::min(chunks, std::max(1, nx / 4));
  const int cx = (nx + chunks - 1) / chunks;
  chunks = (nx + cx - 1) / cx;
  dim3 grid(tiles, chunks, nb), block(kZP, kBY / YPT);
  if (nparts) *nparts = tiles * chunks;
  kern<<<grid, block, G::SMEM, s>>>(tm, vm, (T*)out, nx, ny, nz, cx, tiles_z, bstride, (T)coef,
                                    dot_part, device_error_word());
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

template <typename T, int R, bool HAS_V, bool STORE, bool DOT>
int launch_tma_mode(const CUtensorMap& tm, const CUtensorMap& vm, void* out, int nb, int nx, int ny,
                    int nz, int64_t bstride, double coef, double* dot_part, int* nparts,
                    cudaStream_t s) {
  const int rows = g_rows_per_thread.load() ? g_rows_per_thread.load() : kDefaultRows;
  if (rows == 2)
    return launch_tma_rows<T, R, 2, HAS_V, STORE, DOT>(tm, vm, out, nb, nx, ny, nz, bstride, coef,
                                                       dot_part, nparts, s);
  return launch_tma_rows<T, R, 4, HAS_V, STORE, DOT>(tm, vm, out, nb, nx, ny, nz, bstride, coef,
                                                     dot_part, nparts, s);
}
template <typename T, int R>
int launch_tma(const void* psi, const void* V, void* out, int nb, int nx, int ny, int nz,
               int64_t bstride, double coef, double* dot_part, int* nparts, cudaStream_t s) {
  alignas(64) unsigned char tm[128];
  TmaBox box;
  box.rank = 4;
  box.dims[0] = nz;
  box.dims[1] = ny;
  box.dims[2] = nx;
  box.dims[3] = nb;
  box.strides_bytes[0] = (uint64_t)nz * sizeof(T);
  box.strides_bytes[1] = (uint64_t)ny * nz * sizeof(T);
  box.strides_bytes[2] = (uint64_t)bstride * sizeof(T);
  box.box[0] = TmaGeom<T, R>::PW;
  box.box[1] = TmaGeom<T, R>::PH;
  box.box[2] = 1;
  box.box[3] = 1;
  GATO_TRY(encode_tma(tm, sizeof(T) == 8 ? GATO_F64 : GATO_F32, psi, box));
  alignas(64) unsigned char vm[128] = {};
  if (V) {
    TmaBox vb;
    vb.rank = 3;
    vb.dims[0] = nz;
    vb.dims[1] = ny;
    vb.dims[2] = nx;
    vb.strides_bytes[0] = (uint64_t)nz * sizeof(T);
    vb.strides_bytes[1] = (uint64_t)ny * nz * sizeof(T);
    vb.box[0] = kBZ;
    vb.box[1] = kBY;
    vb.box[2] = 1;
    GATO_TRY(encode_tma(vm, sizeof(T) == 8 ? GATO_F64 : GATO_F32, V, vb));
  } else {
    memcpy(vm, tm, sizeof(vm));   // never read without V
  }
  const CUtensorMap& T4 = *reinterpret_cast<const CUtensorMap*>(tm);
  const CUtensorMap& V3 = *reinterpret_cast<const CUtensorMap*>(vm);
  const int mode = (V ? 4 : 0) | (out ? 2 : 0) | (dot_part ? 1 : 0);
#define GATO_TMA_MODE(M, HV, ST, DT)                                                          \
  case M:                                                                                    \
    return launch_tma_mode<T, R, HV, ST, DT>(T4, V3, out, nb, nx, ny, nz, bstride, coef,     \
                                             dot_part, nparts, s);
  switch (mode) {
    GATO_TMA_MODE(1, false, false, true)
    GATO_TMA_MODE(2, false, true, false)
    GATO_TMA_MODE(3, false, true, true)
    GATO_TMA_MODE(5, true, false, true)
    GATO_TMA_MODE(6, true, true, false)
    GATO_TMA_MODE(7, true, true, true)
    default:
      return fail(GATO_EBADARG, "stencil: nothing to compute");
  }
#undef GATO_TMA_MODE
}

template <typename T>
int stencil_typed(const void* psi, const void* V, void* out, int nb, int nx, int ny, int nz,
                  int64_t bstride, double coef, int boundary, int order, double* dot_dev,
                  double dv, cudaStream_t s) {
  const bool tma_ok = boundary == GATO_DIRICHLET && ((uint64_t)nz * sizeof(T)) % 16 == 0 &&
                      ((uint64_t)bstride * sizeof(T)) % 16 == 0 &&
                      ((uintptr_t)psi % 16) == 0 && ((uintptr_t)V % 16) == 0 &&
                      ((uintptr_t)out % 16) == 0 && nb <= 65535;
  double* part = nullptr;
  if (dot_dev) {
    // worst case: generic path uses kRedBlocks partials per batch.
    part = (double*)stream_scratch(s, (size_t)nb * 4096 * sizeof(double));
    if (!part) return fail(GATO_ENOMEM, "stencil: scratch allocation failed");
  }
  if (tma_ok) {
    int nparts = 0;
    if (order == 2)
      GATO_TRY(launch_tma<T, 1>(psi, V, out, nb, nx, ny, nz, bstride, coef, part, &nparts, s));
    else
      GATO_TRY(launch_tma<T, 2>(psi, V, out, nb, nx, ny, nz, bstride, coef, part, &nparts, s));
    if (dot_dev) {
      if (nparts > 4096) return fail(GATO_EUNSUPPORTED, "stencil: too many tiles for dot");
      GATO_TRY(finalize_sums(part, nb, nparts, dv, dot_dev, s));
    }
    return GATO_OK;
  }
  const int64_t n3 = (int64_t)nx * ny * nz;
  unsigned gx = grid_for(n3, 256, dot_dev ? kRedBlocks : 152 * 16);
  dim3 grid(gx, dot_dev ? nb : 1);
  const bool per = boundary == GATO_PERIODIC;
#define GATO_GEN(RR, PP)                                                                  \
  k_stencil_generic<T, RR, PP><<<grid, 256, 0, s>>>((const T*)psi, (const T*)V, (T*)out, nb, \
                                                    nx, ny, nz, bstride, (T)coef, part)
  if (order == 2) {
    if (per) GATO_GEN(1, true);
    else GATO_GEN(1, false);
  } else {
    if (per) GATO_GEN(2, true);
    else GATO_GEN(2, false);
  }
#undef GATO_GEN
  GATO_LAUNCH_TRY();
  if (dot_dev) GATO_TRY(finalize_sums(part, nb, (int)gx, dv, dot_dev, s));
  return GATO_OK;
}

}  // namespace

int stencil_apply(int dtype, const void* psi, const void* V, void* out, int nb, int nx, int ny,
                  int nz, int64_t bstride, double coef, int boundary, int order, double* dot_dev,
                  double dv, cudaStream_t s) {
  if (order != 2 && order != 4)
    return fail(GATO_EBADARG, "Unknown order %d; expected 2 or 4.", order);
  if (boundary != GATO_DIRICHLET && boundary != GATO_PERIODIC)
    return fail(GATO_EBADARG, "Unknown boundary %d; expected 'dirichlet' or 'periodic'.", boundary);
  if (!psi || (!out && !dot_dev) || nb <= 0 || nx <= 0 || ny <= 0 || nz <= 0)
    return fail(GATO_EBADARG, "stencil: bad arguments");
  if (dtype == GATO_F64)
    return stencil_typed<double>(psi, V, out, nb, nx, ny, nz, bstride, coef, boundary, order,
                                 dot_dev, dv, s);
  if (dtype == GATO_F32)
    return stencil_typed<float>(psi, V, out, nb, nx, ny, nz, bstride, coef, boundary, order,
                                dot_dev, dv, s);
  return fail(GATO_EBADARG, "bad dtype %d", dtype);
}

int stencil_tune(int rows_per_thread) {
  if (rows_per_thread != 0 && rows_per_thread != 2 && rows_per_thread != 4)
    return fail(GATO_EBADARG, "stencil tune: rows per thread must be 0, 2 or 4, got %d",
                rows_per_thread);
  g_rows_per_thread.store(rows_per_thread);
  return GATO_OK;
}

}  // namespace gato

extern "C" int gato_stencil_tune(int rows_per_thread) {
  return gato::stencil_tune(rows_per_thread);
}

extern "C" int gato_stencil_apply(int dtype, const void* psi, const void* V, void* out, int nb,
                                  int nx, int ny, int nz, double lap_coef, int boundary,
                                  int order, double* dot_dev, double dv, void* stream) {
  return gato::stencil_apply(dtype, psi, V, out, nb, nx, ny, nz, (int64_t)nx * ny * nz, lap_coef,
                             boundary, order, dot_dev, dv, gato::as_stream(stream));
}
