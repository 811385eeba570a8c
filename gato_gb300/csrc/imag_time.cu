// Imaginary-time propagation (solvers/imag_time.py:29-65) and the radial
// density histogram (observables.py:41-59).
//
// One Euler step psi <- (psi - dt H psi) / |psi - dt H psi| is a single
// stencil launch, because psi - dt(-1/2 L psi / h^2 + V psi) =
// (dt / (2 h^2)) L psi + (1 - dt V) psi: the stencil kernel with coefficient
// dt / (2 h^2) and the potential 1 - dt V, followed by the norm reduction and
// one rescaling pass. The step (4 launches) is captured once into a CUDA
// graph on a private stream and replayed n_steps - 1 times; the Rayleigh
// quotients at the logged steps run eagerly between replays. If the capture
// is refused the steps run as plain launches.
#include "common.cuh"
#include "stencil.cuh"

#include <vector>

namespace gato {
namespace {

template <typename T>
__global__ void k_one_minus_dt_v(const T* __restrict__ V, T* Vp, int64_t n, double dt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    Vp[i] = (T)(1.0 - dt * (V ? (double)V[i] : 0.0));
}

// dst = src / sqrt(nsq[0]); src may alias dst
template <typename T>
__global__ void k_scale_rsqrt(const T* src, T* dst, int64_t n, const double* nsq) {
  __shared__ double sc;   // one FP64 reciprocal square root per block
  if (threadIdx.x == 0) sc = 1.0 / sqrt(nsq[0]);
  __syncthreads();
  const T s = (T)sc;   // products in the field type (FP64 per element is slow on GB300)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] * s;
}

__global__ void k_div_store(const double* num, const double* den, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = num[0] / den[0];
}

struct ImagState {
  int dtype;
  void* psi;
  void* tmp;
  void* Vp;
  const void* V;
  int N, order, boundary;
  int64_t n3;
  double h, dV, coef;
  double* scal;   // [0] |psi|^2, [1] <psi|H|psi>
};

int launch_1d(int dtype, const void* a, void* b, int64_t n, const double* nsq, cudaStream_t s) {
  const unsigned g = grid_for(n, 256);
  if (dtype == GATO_F64) k_scale_rsqrt<double><<<g, 256, 0, s>>>((const double*)a, (double*)b, n, nsq);
  else k_scale_rsqrt<float><<<g, 256, 0, s>>>((const float*)a, (float*)b, n, nsq);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

// psi <- normalise((dt/(2h^2)) L psi + (1 - dt V) psi)
int step(const ImagState& st, cudaStream_t s) {
  GATO_TRY(stencil_apply(st.dtype, st.psi, st.Vp, st.tmp, 1, st.N, st.N, st.N, st.n3, st.coef,
                         st.boundary, st.order, nullptr, 0.0, s));
  GATO_TRY(dot_impl(st.dtype, st.tmp, st.tmp, st.n3, st.dV, st.scal, s));
  return launch_1d(st.dtype, st.tmp, st.psi, st.n3, st.scal, s);
}

// out = <psi|H|psi> / <psi|psi> (hamiltonian.py:33-35)
int rayleigh(const ImagState& st, double* out, cudaStream_t s) {
  GATO_TRY(stencil_apply(st.dtype, st.psi, st.V, nullptr, 1, st.N, st.N, st.N, st.n3,
                         -0.5 / (st.h * st.h), st.boundary, st.order, st.scal + 1, st.dV, s));
  GATO_TRY(dot_impl(st.dtype, st.psi, st.psi, st.n3, st.dV, st.scal, s));
  k_div_store<<<1, 32, 0, s>>>(st.scal + 1, st.scal, out);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

// Step i is logged when i % log_every == 0 or i == n_steps - 1 (imag_time.py:58-61).
bool logged(int i, int n_steps, int log_every) { return (i % log_every == 0) || (i == n_steps - 1); }

template <typename T>
__global__ void k_radial_hist(const T* __restrict__ re, const T* __restrict__ im, int N, double L, double h,
                              const double* __restrict__ edges, int nb, double dV, double* hist) {
  extern __shared__ double sh_hist[];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sh_hist[b] = 0.0;
  __syncthreads();
  const int64_t n3 = (int64_t)N * N * N;
  const double lo = edges[0], hi = edges[nb];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % N), y = (int)((i / N) % N), x = (int)(i / ((int64_t)N * N));
    const double X = -L / 2 + (x + 0.5) * h, Y = -L / 2 + (y + 0.5) * h, Z = -L / 2 + (z + 0.5) * h;
    const double r = sqrt(X * X + Y * Y + Z * Z);
    if (!(r >= lo && r <= hi)) continue;
    // numpy.histogram's binning: the linear guess, corrected against the
    // actual edges; the last bin is closed on the right.
    int k = (int)((r - lo) / (hi - lo) * nb);
    if (k >= nb) k = nb - 1;
    if (k > 0 && r < edges[k]) --k;
    else if (k < nb - 1 && r >= edges[k + 1]) ++k;
    const double a = (double)re[i], b = im ? (double)im[i] : 0.0;
    atomicAdd(&sh_hist[k], (a * a + b * b) * dV);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (sh_hist[b] != 0.0) atomicAdd(&hist[b], sh_hist[b]);
}

}  // namespace
}  // namespace gato

using namespace gato;

extern "C" int gato_imag_time(int dtype, void* psi, const void* V, int N, double h, int order, int boundary,
                              double dt, int n_steps, int log_every, double* energies_dev, void* stream) {
  if (!psi || N < 1 || h <= 0 || dt <= 0 || n_steps < 0 || log_every < 1 ||
      (n_steps > 0 && !energies_dev))
    return fail(GATO_EBADARG, "gato_imag_time: bad arguments");
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  if (order != 2 && order != 4) return fail(GATO_EBADARG, "Unknown order %d; expected 2 or 4.", order);
  if (boundary != GATO_DIRICHLET && boundary != GATO_PERIODIC)
    return fail(GATO_EBADARG, "Unknown boundary %d; expected 'dirichlet' or 'periodic'.", boundary);
  cudaStream_t user = as_stream(stream);
  const int64_t n3 = (int64_t)N * N * N;
  const size_t es = dtype == GATO_F64 ? 8 : 4;
  const size_t field = (n3 * es + 255) / 256 * 256;

  // A private stream: capture needs a non-legacy stream, and the scratch of
  // the reductions is keyed by stream, so the warm-up step allocates it
  // before the capture.
  cudaStream_t cs = nullptr;
  GATO_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaEvent_t ev = nullptr;
  int rc = GATO_OK;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  do {
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(ev, user) != cudaSuccess || cudaStreamWaitEvent(cs, ev, 0) != cudaSuccess) {
      rc = fail(GATO_ECUDA, "gato_imag_time: stream setup failed");
      break;
    }
    unsigned char* buf = (unsigned char*)stream_scratch(cs, 2 * field + 256, kSlotImagTime);
    // the reduction partials of every call below, sized once so that no
    // later call reallocates a buffer the captured graph points into
    if (!stream_scratch(cs, (size_t)4096 * sizeof(double))) buf = nullptr;
    if (!buf) {
      rc = fail(GATO_ENOMEM, "gato_imag_time: scratch allocation failed");
      break;
    }
    ImagState st{dtype, psi, buf, buf + field, V, N, order, boundary, n3, h, h * h * h,
                 0.5 * dt / (h * h), (double*)(buf + 2 * field)};
    const unsigned g = grid_for(n3, 256);
    if (dtype == GATO_F64) k_one_minus_dt_v<double><<<g, 256, 0, cs>>>((const double*)V, (double*)st.Vp, n3, dt);
    else k_one_minus_dt_v<float><<<g, 256, 0, cs>>>((const float*)V, (float*)st.Vp, n3, dt);
    if ((rc = cudaGetLastError() == cudaSuccess ? GATO_OK : fail(GATO_ECUDA, "k_one_minus_dt_v")) != GATO_OK)
      break;
    count_launch();
    // psi / sqrt(norm_sq(psi)) (imag_time.py:51)
    if ((rc = dot_impl(dtype, psi, psi, n3, st.dV, st.scal, cs)) != GATO_OK) break;
    if ((rc = launch_1d(dtype, psi, psi, n3, st.scal, cs)) != GATO_OK) break;
    int logs = 0;
    for (int i = 0; i < n_steps; ++i) {
      if (i == 0 || !exec) {
        if ((rc = step(st, cs)) != GATO_OK) break;
      } else {
        if (cudaGraphLaunch(exec, cs) != cudaSuccess) {
          rc = fail(GATO_ECUDA, "gato_imag_time: graph launch failed");
          break;
        }
        count_launch();
      }
      if (i == 0 && n_steps > 1) {
        // capture one step; on refusal keep stepping with plain launches
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const int crc = step(st, cs);
          cudaGraph_t gr = nullptr;
          const cudaError_t ce = cudaStreamEndCapture(cs, &gr);
          if (crc == GATO_OK && ce == cudaSuccess && gr &&
              cudaGraphInstantiate(&exec, gr, 0) == cudaSuccess) {
            graph = gr;
          } else {
            if (gr) cudaGraphDestroy(gr);
            exec = nullptr;
          }
          cudaGetLastError();   // a refused capture leaves no sticky error
        }
      }
      if (logged(i, n_steps, log_every)) {
        if ((rc = rayleigh(st, energies_dev + logs, cs)) != GATO_OK) break;
        ++logs;
      }
    }
  } while (false);
  // hand the work back to the caller's stream, then release the private one
  if (ev && cudaEventRecord(ev, cs) == cudaSuccess) cudaStreamWaitEvent(user, ev, 0);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (ev) cudaEventDestroy(ev);
  release_stream_scratch(cs);
  cudaStreamDestroy(cs);
  return rc;
}

extern "C" int gato_radial_density(int dtype, const void* re, const void* im, int N, double L,
                                   const double* edges_host, int n_bins, double* hist_dev, void* stream) {
  if (!re || N < 1 || L <= 0 || !edges_host || n_bins < 1 || !hist_dev || n_bins > 4096)
    return fail(GATO_EBADARG, "gato_radial_density: bad arguments");
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  cudaStream_t s = as_stream(stream);
  double* edges = (double*)stream_scratch(s, (size_t)(n_bins + 1) * sizeof(double));
  if (!edges) return fail(GATO_ENOMEM, "gato_radial_density: scratch allocation failed");
  GATO_CUDA_TRY(cudaMemcpyAsync(edges, edges_host, (n_bins + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
  GATO_CUDA_TRY(cudaMemsetAsync(hist_dev, 0, n_bins * sizeof(double), s));
  const double h = L / N;
  const int64_t n3 = (int64_t)N * N * N;
  const size_t sm = (size_t)n_bins * sizeof(double);
  if (dtype == GATO_F64)
    k_radial_hist<double><<<grid_for(n3, 256, 152 * 4), 256, sm, s>>>((const double*)re, (const double*)im, N, L,
                                                                       h, edges, n_bins, h * h * h, hist_dev);
  else
    k_radial_hist<float><<<grid_for(n3, 256, 152 * 4), 256, sm, s>>>((const float*)re, (const float*)im, N, L, h,
                                                                      edges, n_bins, h * h * h, hist_dev);
  GATO_LAUNCH_TRY();
  // the edges buffer is stream scratch: keep the copy ordered before reuse
  GATO_CUDA_TRY(cudaStreamSynchronize(s));
  return GATO_OK;
}
