// Shared device/host utilities of libgato_cuda (sm_103a only).
#pragma once
#include <initializer_list>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include "../../include/gato.h"

namespace gato {

// ---- errors ------------------------------------------------------------------
int fail(int code, const char* fmt, ...);
const char* last_error();

#define GATO_CUDA_TRY(...)                                                              \
  do {                                                                                  \
    cudaError_t _e = (__VA_ARGS__);                                                     \
    if (_e != cudaSuccess)                                                              \
      return ::gato::fail(_e == cudaErrorMemoryAllocation ? GATO_ENOMEM : GATO_ECUDA,   \
                          "%s failed: %s (%s:%d)", #__VA_ARGS__, cudaGetErrorString(_e), \
                          __FILE__, __LINE__);                                          \
  } while (0)
// Every kernel launch is followed by GATO_LAUNCH_TRY(), which also counts it.
void count_launch();
#define GATO_LAUNCH_TRY()            \
  do {                               \
    ::gato::count_launch();          \
    GATO_CUDA_TRY(cudaGetLastError()); \
  } while (0)
#define GATO_TRY(...)              \
  do {                             \
    int _s = (__VA_ARGS__);        \
    if (_s != GATO_OK) return _s;  \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Per-device error word written by bounded spin-waits (never a trap).
int* device_error_word();

// Per-(device, stream, slot) scratch for reduction partials, grown on demand.
// The first call on a stream may allocate; later calls of the same or
// smaller size do not. Slot 0 serves leaf reductions; a driver that calls
// leaf operations while holding scratch uses its own slot.
enum ScratchSlot { kSlotLeaf = 0, kSlotLanczos = 1, kSlotImagTime = 2, kSlotLanczosSweep = 3, kSlotCount = 4 };
void* stream_scratch(cudaStream_t s, size_t bytes, int slot = kSlotLeaf);
// Raise kernel fn's dynamic shared-memory limit to at least `bytes` on the current device. The
// limit is one setting per kernel shared by every host thread, so it only ever grows (under a
// lock): setting it to each launch's own size would let one thread lower it between another
// thread's setting and launch, which then fails.
int raise_smem_limit(const void* fn, size_t bytes);
// Free every scratch slot of stream s (synchronises s first): for private
// streams that are about to be destroyed.
void release_stream_scratch(cudaStream_t s);
// cudaFree of device memory whose last users may still be queued on some
// stream: waits for the device first, since cudaFree itself only "may"
// synchronise, and memory it returned early could be handed to another
// thread's allocation while those kernels still write it. Null entries are
// skipped; nothing is waited for when all are null.
void free_after_pending(std::initializer_list<void*> ptrs);
// sum_i a_i b_i * scale into out[0] (device), FP64 / float-float accumulation.
int dot_impl(int dtype, const void* a, const void* b, int64_t n, double scale, double* out,
             cudaStream_t s);

// Elementwise launch geometry: a grid-stride loop over n items.
inline unsigned grid_for(int64_t n, int threads, int max_blocks = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b > max_blocks) b = max_blocks;
  if (b < 1) b = 1;
  return (unsigned)b;
}

constexpr int kRedBlocks = 304;     // 2 x 152 SMs: partial sums per reduction
constexpr int kRedThreads = 256;

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

// ---- float-float accumulation (FP32 path reductions) ----------------------------
// Error-free transforms of Knuth (two-sum) and the FMA two-product; the pair
// (hi, lo) carries ~48 significant bits, so FP32 fields reduce without the
// FP64 pipe, which is the scarce unit on GB300.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ void ff_add(FF& s, float x) {
  float t = s.hi + x;
  float bp = t - s.hi;
  float err = (s.hi - (t - bp)) + (x - bp);
  s.hi = t;
  s.lo += err;
}
__device__ __forceinline__ void ff_add_prod(FF& s, float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  ff_add(s, p);
  s.lo += e;
}
__device__ __forceinline__ double ff_value(const FF& s) { return (double)s.hi + (double)s.lo; }

// Generic per-thread accumulator: double for FP64 fields, float-float for FP32.
template <typename T> struct Acc;
template <> struct Acc<double> {
  double v = 0.0;
  __device__ __forceinline__ void add_prod(double a, double b) { v = fma(a, b, v); }
  __device__ __forceinline__ void add(double a) { v += a; }
  __device__ __forceinline__ double value() const { return v; }
};
template <> struct Acc<float> {
  FF s{0.f, 0.f};
  __device__ __forceinline__ void add_prod(float a, float b) { ff_add_prod(s, a, b); }
  __device__ __forceinline__ void add(float a) { ff_add(s, a); }
  __device__ __forceinline__ double value() const { return ff_value(s); }
};

// Block-wide sum of a double; every thread gets the result. `sh` holds
// >= 32 doubles.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  int lane = tid & 31, warp = tid >> 5;
  int nw = (nt + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = (tid < nw) ? sh[tid] : 0.0;
  if (warp == 0) t = warp_sum(t);
  if (tid == 0) sh[0] = t;
  __syncthreads();
  double r = sh[0];
  __syncthreads();
  return r;
}

// Reduce partials[q * nparts + i] over i (fixed order) into out[q] * scale.
// Launched with one block per q.
__global__ void k_finalize_sums(const double* partials, int nparts, double scale, double* out);
int finalize_sums(const double* partials, int nq, int nparts, double scale, double* out,
                  cudaStream_t s);

// ---- TMA tensor-map encoding (driver entry point, no libcuda link) ----------
struct TmaBox {
  int rank;
  uint64_t dims[5];
  uint64_t strides_bytes[4];  // dims 1..rank-1
  uint32_t box[5];
};
// Encodes a tiled tensor map with zero out-of-bounds fill into `out128`
// (a 128-byte CUtensorMap).
int encode_tma(void* out128, int dtype, const void* base, const TmaBox& b);

}  // namespace gato
