// Finite-difference Laplacian / Hamiltonian apply (operators.py:40-130,
// hamiltonian.py:25-31).
//
// Hot path (Dirichlet, 16-byte aligned rows): each CTA owns a 16 (y) x 32 (z)
// column of the grid and marches along x through a chunk of planes. One
// elected thread streams (16+2R) x (32+2A) halo planes into an 8-slot
// shared-memory ring with TMA (cp.async.bulk.tensor, mbarrier completion);
// the tensor map's zero out-of-bounds fill is exactly the reference's zero
// padding, so no boundary branches exist. x-neighbours live in a per-thread
// register queue, y/z neighbours are read from the centre plane in shared
// memory. V and the output are plain coalesced accesses. HBM-bound: the
// algorithmic traffic is 3 N^3 s bytes (psi, V, out).
#include <cuda.h>

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
constexpr int kBY = 16;       // tile height along y
constexpr int kTY = 8;        // thread rows: each thread owns kBY/kTY points
constexpr int kYPT = kBY / kTY;
constexpr int kSlots = 8;     // plane ring depth

template <typename T, int R>
struct TmaGeom {
  static constexpr int A = 16 / (int)sizeof(T);  // z halo, rounded to 16 bytes
  static constexpr int PW = kBZ + 2 * A;
  static constexpr int PH = kBY + 2 * R;
  static constexpr int BOX_BYTES = PW * PH * (int)sizeof(T);
  static constexpr int SLOT_BYTES = (BOX_BYTES + 127) / 128 * 128;
  static constexpr int SMEM = kSlots * SLOT_BYTES + kSlots * 8 + 128;
};

template <typename T, int R>
__global__ void __launch_bounds__(kBZ* kTY)
    k_stencil_tma(const __grid_constant__ CUtensorMap tmap, const T* __restrict__ V,
                  T* __restrict__ out, int nx, int ny, int nz, int cx, int tiles_z,
                  int64_t bstride, T coef, double* dot_part, int* err) {
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

  auto issue = [&](int q) {
    int s = q % kSlots;
    mbar_expect_tx(&bars[s], G::BOX_BYTES);
    tma_load_4d(smem + s * G::SLOT_BYTES, &tmap, &bars[s], z0 - G::A, y0 - R, xs - R + q, b);
  };
  if (tid == 0) {
    int n0 = P < kSlots ? P : kSlots;
    for (int q = 0; q < n0; ++q) issue(q);
  }

  T xq[kYPT][2 * R + 1];
#pragma unroll
  for (int k = 0; k < kYPT; ++k)
#pragma unroll
    for (int r = 0; r < 2 * R + 1; ++r) xq[k][r] = (T)0;

  Acc<T> acc;
  const int gz = z0 + tz;
  // V of the next output plane, loaded one iteration ahead so its latency
  // overlaps the barrier and the plane wait.
  T vn[kYPT];
  auto load_v = [&](int xo) {
#pragma unroll
    for (int k = 0; k < kYPT; ++k) {
      const int gy = y0 + ty + k * kTY;
      vn[k] = (V && xo < xe && gy < ny && gz < nz) ? V[((int64_t)xo * ny + gy) * nz + gz] : (T)0;
    }
  };
  load_v(xs);
  for (int q = 0; q < P; ++q) {
    const int s = q % kSlots;
    mbar_wait_bounded(&bars[s], (uint32_t)((q / kSlots) & 1), err, 101);
    const T* pl = reinterpret_cast<const T*>(smem + s * G::SLOT_BYTES);
#pragma unroll
    for (int k = 0; k < kYPT; ++k) {
      const int y = ty + k * kTY;
#pragma unroll
      for (int r = 0; r < 2 * R; ++r) xq[k][r] = xq[k][r + 1];
      xq[k][2 * R] = pl[(y + R) * G::PW + (tz + G::A)];
    }
    if (q >= 2 * R) {
      const int xo = xs + q - 2 * R;
      const T* pc = reinterpret_cast<const T*>(smem + ((q - R) % kSlots) * G::SLOT_BYTES);
#pragma unroll
      for (int k = 0; k < kYPT; ++k) {
        const int y = ty + k * kTY;
        const int gy = y0 + y;
        const int idx = (y + R) * G::PW + (tz + G::A);
        const T ctr = xq[k][R];
        T s1 = xq[k][R - 1] + xq[k][R + 1] + pc[idx - G::PW] + pc[idx + G::PW] + pc[idx - 1] +
               pc[idx + 1];
        T s2 = (T)0;
        if constexpr (R == 2)
          s2 = xq[k][0] + xq[k][4] + pc[idx - 2 * G::PW] + pc[idx + 2 * G::PW] + pc[idx - 2] +
               pc[idx + 2];
        T val = coef * lap_combine<T>(ctr, s1, s2, c, R);
        if (gy < ny && gz < nz) {
          const int64_t gi = (int64_t)b * bstride + ((int64_t)xo * ny + gy) * nz + gz;
          if (V) val += vn[k] * ctr;
          if (out) out[gi] = val;
          if (dot_part) acc.add_prod(ctr, val);
        }
      }
      load_v(xo + 1);
    }
    __syncthreads();  // every thread is done with plane q - R
    if (tid == 0 && q >= R && q - R + kSlots < P) issue(q - R + kSlots);
  }
  if (dot_part) {
    double v = block_sum(acc.value(), sh);
    if (tid == 0)
      dot_part[(int64_t)b * gridDim.x * gridDim.y + (int64_t)blockIdx.y * gridDim.x + blockIdx.x] =
          v;
  }
}

template <typename T, int R>
int launch_tma(const void* psi, const void* V, void* out, int nb, int nx, int ny, int nz,
               int64_t bstride, double coef, double* dot_part, int* nparts, cudaStream_t s) {
  using G = TmaGeom<T, R>;
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
  box.box[0] = G::PW;
  box.box[1] = G::PH;
  box.box[2] = 1;
  box.box[3] = 1;
  GATO_TRY(encode_tma(tm, sizeof(T) == 8 ? GATO_F64 : GATO_F32, psi, box));
  const int tiles_z = (nz + kBZ - 1) / kBZ, tiles_y = (ny + kBY - 1) / kBY;
  const int tiles = tiles_z * tiles_y;
  // Chunk length along x: enough CTAs to fill 152 SMs about three deep,
  // but no chunk shorter than 8 planes (the 2R halo planes are overhead).
  int cx = nx;
  while (cx > 8 && (int64_t)tiles * ((nx + cx - 1) / cx) * nb < 3 * 152) cx = (cx + 1) / 2;
  const int chunks = (nx + cx - 1) / cx;
  GATO_CUDA_TRY(cudaFuncSetAttribute(k_stencil_tma<T, R>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM));
  dim3 grid(tiles, chunks, nb), block(kBZ, kTY);
  if (nparts) *nparts = tiles * chunks;
  k_stencil_tma<T, R><<<grid, block, G::SMEM, s>>>(
      *reinterpret_cast<const CUtensorMap*>(tm), (const T*)V, (T*)out, nx, ny, nz, cx, tiles_z,
      bstride, (T)coef, dot_part, device_error_word());
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

template <typename T>
int stencil_typed(const void* psi, const void* V, void* out, int nb, int nx, int ny, int nz,
                  int64_t bstride, double coef, int boundary, int order, double* dot_dev,
                  double dv, cudaStream_t s) {
  const bool tma_ok = boundary == GATO_DIRICHLET && ((uint64_t)nz * sizeof(T)) % 16 == 0 &&
                      ((uint64_t)bstride * sizeof(T)) % 16 == 0 &&
                      ((uintptr_t)psi % 16) == 0 && nb <= 65535;
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
