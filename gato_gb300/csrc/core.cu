// Library core: error state, device error word, stream scratch, reductions,
// TMA encoding, and the grid.py reductions of the C ABI.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

namespace gato {

static thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
const char* last_error() { return g_last_error.c_str(); }

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static std::mutex g_mu;
static std::map<int, int*> g_err_words;
static std::map<std::pair<std::pair<int, int>, cudaStream_t>, std::pair<void*, size_t>> g_scratch;

int* device_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_err_words.find(dev);
  if (it != g_err_words.end()) return it->second;
  int* p = nullptr;
  if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
  // cleared on the legacy stream and waited for: kernels on non-blocking streams write it next
  if (cudaMemsetAsync(p, 0, sizeof(int), cudaStreamLegacy) != cudaSuccess ||
      cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess)
    return nullptr;
  g_err_words[dev] = p;
  return p;
}

void* stream_scratch(cudaStream_t s, size_t bytes, int slot) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  auto& e = g_scratch[{{dev, slot}, s}];
  if (e.second >= bytes) return e.first;
  if (e.first) {
    // the old buffer's users are this stream's queued kernels: let them finish first
    cudaStreamSynchronize(s);
    cudaFree(e.first);
  }
  size_t sz = bytes < (1u << 20) ? (1u << 20) : bytes;
  void* p = nullptr;
  if (cudaMalloc(&p, sz) != cudaSuccess) {
    e = {nullptr, 0};
    return nullptr;
  }
  e = {p, sz};
  return p;
}

int raise_smem_limit(const void* fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> cur;
  int dev = 0;
  GATO_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& c = cur[{dev, fn}];
  if (bytes > c) {
    GATO_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    c = bytes;
  }
  return GATO_OK;
}

void free_after_pending(std::initializer_list<void*> ptrs) {
  bool any = false;
  for (void* p : ptrs) any = any || p != nullptr;
  if (!any) return;
  cudaDeviceSynchronize();
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

void release_stream_scratch(cudaStream_t s) {
  cudaStreamSynchronize(s);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(g_mu);
  for (int slot = 0; slot < kSlotCount; ++slot) {
    auto it = g_scratch.find({{dev, slot}, s});
    if (it == g_scratch.end()) continue;
    if (it->second.first) cudaFree(it->second.first);
    g_scratch.erase(it);
  }
}

__global__ void k_finalize_sums(const double* partials, int nparts, double scale, double* out) {
  __shared__ double sh[32];
  const double* p = partials + (size_t)blockIdx.x * nparts;
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += p[i];
  v = block_sum(v, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = v * scale;
}

int finalize_sums(const double* partials, int nq, int nparts, double scale, double* out,
                  cudaStream_t s) {
  if (nq <= 0) return GATO_OK;
  k_finalize_sums<<<nq, 256, 0, s>>>(partials, nparts, scale, out);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int encode_tma(void* out128, int dtype, const void* base, const TmaBox& b) {
  if (!g_encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    GATO_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn)
      return fail(GATO_ECUDA, "cuTensorMapEncodeTiled entry point unavailable");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  cuuint64_t dims[5], strides[4];
  cuuint32_t box[5], estr[5];
  for (int i = 0; i < b.rank; ++i) {
    dims[i] = b.dims[i];
    box[i] = b.box[i];
    estr[i] = 1;
  }
  for (int i = 0; i + 1 < b.rank; ++i) strides[i] = b.strides_bytes[i];
  CUresult r = g_encode(reinterpret_cast<CUtensorMap*>(out128),
                        dtype == GATO_F64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                          : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                        (cuuint32_t)b.rank, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(GATO_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GATO_OK;
}

// ---- grid.py reductions --------------------------------------------------------

template <typename T>
__global__ void k_dot_partials(const T* __restrict__ a, const T* __restrict__ b, int64_t n,
                               double* partials) {
  __shared__ double sh[32];
  Acc<T> acc;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    if (b) acc.add_prod(a[i], b[i]);
    else acc.add(a[i]);
  }
  double v = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// sum_i a_i w_i b_i: the <psi|V|psi> of observables.py:26-30
template <typename T>
__global__ void k_wdot_partials(const T* __restrict__ a, const T* __restrict__ w, const T* __restrict__ b,
                                int64_t n, double* partials) {
  __shared__ double sh[32];
  Acc<T> acc;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    acc.add_prod(a[i] * w[i], b[i]);
  double v = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

template <typename T>
__global__ void k_normalize(T* a, int64_t n, const double* nsq) {
  __shared__ double sc;   // one FP64 reciprocal square root per block
  if (threadIdx.x == 0) sc = 1.0 / sqrt(nsq[0]);
  __syncthreads();
  const T s = (T)sc;   // products in the field type (FP64 per element is slow on GB300)
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    a[i] = a[i] * s;
}

template <typename T>
__global__ void k_density(const T* __restrict__ orb, int n, int64_t npts, T* rho) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += stride) {
    T s = 0;
    for (int k = 0; k < n; ++k) {
      T v = orb[(int64_t)k * npts + i];
      s += v * v;
    }
    rho[i] = (T)2 * s;
  }
}

template <typename T>
__global__ void k_mix(T* rho, const T* __restrict__ rnew, int64_t npts, double a) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += stride)
    rho[i] = (T)(a * (double)rnew[i] + (1.0 - a) * (double)rho[i]);
}

}  // namespace gato

using namespace gato;

extern "C" int gato_version(void) { return 1; }

extern "C" long long gato_launch_count(void) { return g_launches.load(); }

extern "C" int gato_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return GATO_EBADARG;
  strncpy(buf, last_error(), len - 1);
  buf[len - 1] = 0;
  return GATO_OK;
}

extern "C" int gato_device_status(int* status_out, void* stream) {
  int* w = device_error_word();
  if (!w) return fail(GATO_ECUDA, "device error word unavailable");
  int v = 0;
  GATO_CUDA_TRY(cudaMemcpyAsync(&v, w, sizeof(int), cudaMemcpyDeviceToHost, as_stream(stream)));
  GATO_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  GATO_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(int), as_stream(stream)));
  if (status_out) *status_out = v;
  return GATO_OK;
}

namespace gato {
int dot_impl(int dtype, const void* a, const void* b, int64_t n, double scale, double* out,
             cudaStream_t s) {
  if (n <= 0 || !a || !out) return fail(GATO_EBADARG, "gato_dot: bad arguments");
  double* part = (double*)stream_scratch(s, kRedBlocks * sizeof(double));
  if (!part) return fail(GATO_ENOMEM, "gato_dot: scratch allocation failed");
  int nb = (int)grid_for(n, kRedThreads, kRedBlocks);
  if (dtype == GATO_F64)
    k_dot_partials<double><<<nb, kRedThreads, 0, s>>>((const double*)a, (const double*)b, n, part);
  else
    k_dot_partials<float><<<nb, kRedThreads, 0, s>>>((const float*)a, (const float*)b, n, part);
  GATO_LAUNCH_TRY();
  return finalize_sums(part, 1, nb, scale, out, s);
}
}  // namespace gato

extern "C" int gato_dot(int dtype, const void* a, const void* b, int64_t n, double scale,
                        double* out_dev, void* stream) {
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  return dot_impl(dtype, a, b, n, scale, out_dev, as_stream(stream));
}

extern "C" int gato_dot_weighted(int dtype, const void* a, const void* w, const void* b, int64_t n,
                                 double scale, double* out_dev, void* stream) {
  if (!a || !w || !b || !out_dev || n <= 0) return fail(GATO_EBADARG, "gato_dot_weighted: bad arguments");
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  cudaStream_t s = as_stream(stream);
  double* part = (double*)stream_scratch(s, kRedBlocks * sizeof(double));
  if (!part) return fail(GATO_ENOMEM, "gato_dot_weighted: scratch allocation failed");
  const int nb = (int)grid_for(n, kRedThreads, kRedBlocks);
  if (dtype == GATO_F64)
    k_wdot_partials<double><<<nb, kRedThreads, 0, s>>>((const double*)a, (const double*)w, (const double*)b,
                                                        n, part);
  else
    k_wdot_partials<float><<<nb, kRedThreads, 0, s>>>((const float*)a, (const float*)w, (const float*)b, n,
                                                       part);
  GATO_LAUNCH_TRY();
  return finalize_sums(part, 1, nb, scale, out_dev, s);
}

extern "C" int gato_normalize(int dtype, void* a, int64_t n, const double* nsq, void* stream) {
  if (!a || !nsq || n <= 0) return fail(GATO_EBADARG, "gato_normalize: bad arguments");
  cudaStream_t s = as_stream(stream);
  unsigned g = grid_for(n, 256);
  if (dtype == GATO_F64) k_normalize<double><<<g, 256, 0, s>>>((double*)a, n, nsq);
  else k_normalize<float><<<g, 256, 0, s>>>((float*)a, n, nsq);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

extern "C" int gato_density(int dtype, const void* orb, int n, int64_t npts, void* rho,
                            void* stream) {
  if (!orb || !rho || n <= 0 || npts <= 0) return fail(GATO_EBADARG, "gato_density: bad arguments");
  cudaStream_t s = as_stream(stream);
  unsigned g = grid_for(npts, 256);
  if (dtype == GATO_F64) k_density<double><<<g, 256, 0, s>>>((const double*)orb, n, npts, (double*)rho);
  else k_density<float><<<g, 256, 0, s>>>((const float*)orb, n, npts, (float*)rho);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

extern "C" int gato_mix(int dtype, void* rho, const void* rnew, int64_t npts, double a,
                        void* stream) {
  if (!rho || !rnew || npts <= 0) return fail(GATO_EBADARG, "gato_mix: bad arguments");
  cudaStream_t s = as_stream(stream);
  unsigned g = grid_for(npts, 256);
  if (dtype == GATO_F64) k_mix<double><<<g, 256, 0, s>>>((double*)rho, (const double*)rnew, npts, a);
  else k_mix<float><<<g, 256, 0, s>>>((float*)rho, (const float*)rnew, npts, a);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

namespace gato {
template <typename T>
__global__ void k_axpby(const T* __restrict__ x, const T* __restrict__ y, T* out, int64_t n, double a,
                        double b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (T)(a * (double)x[i] + b * (double)y[i]);
}
template <typename T>
__global__ void k_field_sum(const T* __restrict__ f, int nf, int64_t n, T* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    T s = 0;
    for (int k = 0; k < nf; ++k) s += f[(int64_t)k * n + i];
    out[i] = s;
  }
}
}  // namespace gato

extern "C" int gato_axpby(int dtype, const void* x, const void* y, void* out, int64_t n, double a,
                          double b, void* stream) {
  if (!x || !y || !out || n <= 0) return fail(GATO_EBADARG, "gato_axpby: bad arguments");
  cudaStream_t s = as_stream(stream);
  unsigned g = grid_for(n, 256);
  if (dtype == GATO_F64) k_axpby<double><<<g, 256, 0, s>>>((const double*)x, (const double*)y, (double*)out, n, a, b);
  else k_axpby<float><<<g, 256, 0, s>>>((const float*)x, (const float*)y, (float*)out, n, a, b);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

extern "C" int gato_field_sum(int dtype, const void* fields, int nf, int64_t n, void* out, void* stream) {
  if (!fields || !out || nf < 1 || n <= 0) return fail(GATO_EBADARG, "gato_field_sum: bad arguments");
  cudaStream_t s = as_stream(stream);
  unsigned g = grid_for(n, 256);
  if (dtype == GATO_F64) k_field_sum<double><<<g, 256, 0, s>>>((const double*)fields, nf, n, (double*)out);
  else k_field_sum<float><<<g, 256, 0, s>>>((const float*)fields, nf, n, (float*)out);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

namespace gato {
template <typename S, typename D>
__global__ void k_convert(const S* __restrict__ src, D* dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (D)src[i];
}
}  // namespace gato

extern "C" int gato_convert(int src_dtype, const void* src, int dst_dtype, void* dst, int64_t n,
                            void* stream) {
  if (!src || !dst || n <= 0) return fail(GATO_EBADARG, "gato_convert: bad arguments");
  cudaStream_t s = as_stream(stream);
  const unsigned g = grid_for(n, 256);
  if (src_dtype == GATO_F64 && dst_dtype == GATO_F32)
    k_convert<double, float><<<g, 256, 0, s>>>((const double*)src, (float*)dst, n);
  else if (src_dtype == GATO_F32 && dst_dtype == GATO_F64)
    k_convert<float, double><<<g, 256, 0, s>>>((const float*)src, (double*)dst, n);
  else if (src_dtype == dst_dtype)
    GATO_CUDA_TRY(cudaMemcpyAsync(dst, src, n * (src_dtype == GATO_F64 ? 8 : 4), cudaMemcpyDeviceToDevice, s));
  else
    return fail(GATO_EBADARG, "gato_convert: bad dtypes %d -> %d", src_dtype, dst_dtype);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}
