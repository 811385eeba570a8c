// Finite-difference Laplacian / Hamiltonian apply (operators.py:40-130,
// hamiltonian.py:25-31).
//
// Hot path (Dirichlet, 16-byte aligned rows): each CTA owns a 32 (y) x 32 (z)
// column of the grid and marches along x through a chunk of planes. One
// elected thread streams (16+2R) x (32+2A) halo planes into an 8-slot
// shared-memory ring with TMA (cp.async.bulk.tensor, mbarrier completion);
// the tensor map's zero out-of-bounds fill is exactly the reference's zero
// padding, so no boundary branches exist. x-neighbours live in a per-thread
// register queue, y/z neighbours are read from the centre plane in shared
// memory. The 16 x 32 V tile of each centre plane rides in the same ring slot
// (a second tensor map, same mbarrier), so V arrives with the ring's
// look-ahead instead of one DRAM round trip per plane; the output is a plain
// coalesced store. HBM-bound: the algorithmic traffic is 3 N^3 s bytes
// (psi, V, out).
#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstring>

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
constexpr int kBZ = 32;       // tile width along z (one warp)
constexpr int kBY = 32;       // tile height along y
constexpr int kTY = 8;        // thread rows; each thread owns kYPT consecutive y rows
constexpr int kYPT = kBY / kTY;
constexpr int kSlots = 6;     // plane ring depth: 3 planes of look-ahead, 3 FP32 (2 FP64) CTAs per SM

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

// One CTA: a kBY x kBZ column of one field, planes [xs, xs + cx) along x.
// Plane q of the chunk is x = xs - R + q and sits in ring slot q % kSlots; it
// feeds the x register queue at iteration q and is the centre plane at
// iteration q + R, after which its slot is refilled with plane q + kSlots.
// The plane loop is unrolled by the ring depth, so slot addresses are
// immediates and the queue shifts are register renames. Each thread owns
// rows yt .. yt + kYPT - 1 at z = tz: its y neighbours are its own queue
// centres plus 2R halo rows, its z neighbours are shared-memory reads.
template <typename T, int R, bool HAS_V, bool STORE, bool DOT>
__global__ void __launch_bounds__(kBZ* kTY)
    k_stencil_tma(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap vmap,
                  T* __restrict__ out, int nx, int ny, int nz, int cx, int tiles_z, int64_t bstride,
                  T coef, double* dot_part, int* err) {
  using G = TmaGeom<T, R>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem =
      (unsigned char*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kSlots * G::SLOT_BYTES);
  __shared__ double sh[32];

  const StencilCoef<T> c = coefs<T>(R == 1 ? 2 : 4);
  const int tz = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * kBZ + tz;
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

  const int yt = ty * kYPT;
  const int gz = z0 + tz;
  unsigned live = 0;
#pragma unroll
  for (int k = 0; k < kYPT; ++k)
    if (gz < nz && y0 + yt + k < ny) live |= 1u << k;
  T* obase = nullptr;
  if (STORE) obase = out + (int64_t)b * bstride + ((int64_t)xs * ny + (y0 + yt)) * nz + gz;
  const int64_t pstride = (int64_t)ny * nz;
  const int cidx = (yt + R) * G::PW + tz + G::A;   // this thread's first row, centre column

  T xq[kYPT][2 * R + 1];
#pragma unroll
  for (int k = 0; k < kYPT; ++k)
#pragma unroll
    for (int r = 0; r < 2 * R + 1; ++r) xq[k][r] = (T)0;
  Acc<T> acc;
  bool bad = false;
  int q = 0;
  for (int qb = 0; qb < P && !bad; qb += kSlots) {
#pragma unroll
    for (int j = 0; j < kSlots; ++j) {
      q = qb + j;
      if (q >= P) break;
      if (!mbar_wait_bounded(&bars[j], (uint32_t)((qb / kSlots) & 1), err, 101)) bad = true;
      const T* pl = reinterpret_cast<const T*>(smem + j * G::SLOT_BYTES);
#pragma unroll
      for (int k = 0; k < kYPT; ++k) {
#pragma unroll
        for (int r = 0; r < 2 * R; ++r) xq[k][r] = xq[k][r + 1];
        xq[k][2 * R] = pl[cidx + k * G::PW];
      }
      if (q >= 2 * R) {
        const int cs = (j + kSlots - R) % kSlots;   // compile-time after unrolling
        const T* pc = reinterpret_cast<const T*>(smem + cs * G::SLOT_BYTES);
        const T* pv = reinterpret_cast<const T*>(smem + cs * G::SLOT_BYTES + G::V_OFF);
        T col[kYPT + 2 * R];
#pragma unroll
        for (int i = 0; i < R; ++i) {
          col[i] = pc[cidx + (i - R) * G::PW];
          col[R + kYPT + i] = pc[cidx + (kYPT + i) * G::PW];
        }
#pragma unroll
        for (int k = 0; k < kYPT; ++k) col[R + k] = xq[k][R];
        T* op = STORE ? obase + (int64_t)(q - 2 * R) * pstride : nullptr;
#pragma unroll
        for (int k = 0; k < kYPT; ++k) {
          const int idx = cidx + k * G::PW;
          const T ctr = xq[k][R];
          T s1 = xq[k][R - 1] + xq[k][R + 1] + col[R + k - 1] + col[R + k + 1] + pc[idx - 1] +
                 pc[idx + 1];
          T s2 = (T)0;
          if constexpr (R == 2)
            s2 = xq[k][0] + xq[k][4] + col[k] + col[k + 4] + pc[idx - 2] + pc[idx + 2];
          T val = coef * lap_combine<T>(ctr, s1, s2, c, R);
          if constexpr (HAS_V) val += pv[(yt + k) * kBZ + tz] * ctr;
          if (live & (1u << k)) {
            if constexpr (STORE) op[k * nz] = val;
            if constexpr (DOT) acc.add_prod(ctr, val);
          }
        }
      }
      // every thread is done with plane q - R; a timed-out wait anywhere stops the CTA
      if (__syncthreads_or(bad)) {
        bad = true;
        break;
      }
      if (tid == 0 && q >= R && q - R + kSlots < P) {
        issue(q - R + kSlots);
        ++issued;
      }
    }
  }
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

// Resident CTAs of a kernel on the whole GPU (occupancy x SMs).
template <typename K>
int resident_ctas(K kernel, int smem) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBZ * kTY, smem) != cudaSuccess ||
      per <= 0)
    return 152;
  return per * sms;
}

template <typename T, int R, bool HAS_V, bool STORE, bool DOT>
int launch_tma_mode(const CUtensorMap& tm, const CUtensorMap& vm, void* out, int nb, int nx, int ny,
                    int nz, int64_t bstride, double coef, double* dot_part, int* nparts,
                    cudaStream_t s) {
  using G = TmaGeom<T, R>;
  auto kern = k_stencil_tma<T, R, HAS_V, STORE, DOT>;
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
  static const int cap = resident_ctas(kern, G::SMEM);   // one value per instantiation
  int chunks = (int)std::max<int64_t>(1, cap / ((int64_t)tiles * nb));
  chunks = std::min(chunks, std::max(1, nx / 4));
  const int cx = (nx + chunks - 1) / chunks;
  chunks = (nx + cx - 1) / cx;
  dim3 grid(tiles, chunks, nb), block(kBZ, kTY);
  if (nparts) *nparts = tiles * chunks;
  kern<<<grid, block, G::SMEM, s>>>(tm, vm, (T*)out, nx, ny, nz, cx, tiles_z, bstride, (T)coef,
                                    dot_part, device_error_word());
  GATO_LAUNCH_TRY();
  return GATO_OK;
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
                      ((uintptr_t)psi % 16) == 0 && ((uintptr_t)V % 16) == 0 && nb <= 65535;
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

}  // namespace gato

extern "C" int gato_stencil_apply(int dtype, const void* psi, const void* V, void* out, int nb,
                                  int nx, int ny, int nz, double lap_coef, int boundary,
                                  int order, double* dot_dev, double dv, void* stream) {
  return gato::stencil_apply(dtype, psi, V, out, nb, nx, ny, nz, (int64_t)nx * ny * nz, lap_coef,
                             boundary, order, dot_dev, dv, gato::as_stream(stream));
}
