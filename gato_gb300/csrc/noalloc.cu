// gato_dot_noalloc: the grid inner product without any device allocation.
//
// Some callers cannot call cudaMalloc: hosts that hand the GPU a fixed memory
// budget through their own allocator and forbid the CUDA runtime's (an
// embedding framework that owns every byte of device memory), and
// latency-critical threads that must not block in the driver (cudaMalloc may
// synchronise the device and takes driver locks). gato_dot obtains its
// partial sums from per-stream scratch that is allocated on first use; this
// variant keeps them in a file-scope __device__ array instead. That array
// (kNoAllocChunks doubles, 512 KiB) exists on every GPU that loads the
// library until the process exits.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress (the host-side name of
// a __device__ variable is only a stand-in, never a device pointer) and caches
// it per device. Every later call allocates nothing and takes no lock.
//
// Limits and sharing: one partial sum per 2048-element chunk, so n may not
// exceed kNoAllocChunks * 2048 = 2^27 elements (a 512^3 grid); larger n is
// rejected with GATO_EBADARG before any device work. All calls share the one
// array: any two calls whose kernels can run at the same time on the GPU
// (different streams, or different host threads without ordering) race on it
// and must be serialised by the caller. Each call overwrites every partial it
// reads, so nothing needs clearing between calls.
#include <atomic>
#include <map>
#include <mutex>

#include "common.cuh"

namespace gato {
namespace {

constexpr int kNoAllocChunks = 65536;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocEPT = 8;
constexpr int64_t kNoAllocChunk = (int64_t)kNoAllocThreads * kNoAllocEPT;   // 2048

__device__ __align__(256) double g_noalloc_partials[kNoAllocChunks];

// device -> address of g_noalloc_partials: a lock-free slot per device id
// below kNoAllocDevs (set once, read on every call), a locked map beyond.
constexpr int kNoAllocDevs = 64;
std::atomic<double*> g_noalloc_slot[kNoAllocDevs];
std::mutex g_noalloc_mu;
std::map<int, double*> g_noalloc_addr;

int noalloc_partials(double** out) {
  int dev = 0;
  GATO_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < kNoAllocDevs) {
    double* p = g_noalloc_slot[dev].load(std::memory_order_acquire);
    if (p) {
      *out = p;
      return GATO_OK;
    }
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  auto it = g_noalloc_addr.find(dev);
  double* p = nullptr;
  if (it != g_noalloc_addr.end()) {
    p = it->second;
  } else {
    GATO_CUDA_TRY(cudaGetSymbolAddress((void**)&p, g_noalloc_partials));
    g_noalloc_addr[dev] = p;
  }
  if (dev >= 0 && dev < kNoAllocDevs) g_noalloc_slot[dev].store(p, std::memory_order_release);
  *out = p;
  return GATO_OK;
}

// part[chunk] = sum of a*b (or a) over one 2048-element chunk
template <typename T>
__global__ void __launch_bounds__(kNoAllocThreads)
    k_dot_chunks(const T* __restrict__ a, const T* __restrict__ b, int64_t n, double* part) {
  __shared__ double sh[32];
  Acc<T> acc;
  const int64_t base = (int64_t)blockIdx.x * kNoAllocChunk;
#pragma unroll
  for (int e = 0; e < kNoAllocEPT; ++e) {
    const int64_t i = base + e * kNoAllocThreads + threadIdx.x;
    if (i < n) {
      if (b) acc.add_prod(a[i], b[i]);
      else acc.add(a[i]);
    }
  }
  const double v = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

}  // namespace
}  // namespace gato

using namespace gato;

extern "C" int gato_dot_noalloc(int dtype, const void* a, const void* b, int64_t n, double scale,
                                double* out_dev, void* stream) {
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  if (!a || !out_dev || n <= 0) return fail(GATO_EBADARG, "gato_dot_noalloc: bad arguments");
  const int64_t nchunks = (n + kNoAllocChunk - 1) / kNoAllocChunk;
  if (nchunks > kNoAllocChunks)
    return fail(GATO_EBADARG,
                "gato_dot_noalloc: n = %lld exceeds the maximum of %lld elements (the static "
                "scratch holds %d partial sums of %lld elements each); use gato_dot",
                (long long)n, (long long)kNoAllocChunks * kNoAllocChunk, kNoAllocChunks,
                (long long)kNoAllocChunk);
  double* part = nullptr;
  GATO_TRY(noalloc_partials(&part));
  cudaStream_t s = as_stream(stream);
  if (dtype == GATO_F64)
    k_dot_chunks<double><<<(unsigned)nchunks, kNoAllocThreads, 0, s>>>((const double*)a, (const double*)b, n, part);
  else
    k_dot_chunks<float><<<(unsigned)nchunks, kNoAllocThreads, 0, s>>>((const float*)a, (const float*)b, n, part);
  GATO_LAUNCH_TRY();
  return finalize_sums(part, 1, (int)nchunks, scale, out_dev, s);
}
