// Internal entry of the stencil kernels (used by the operator and the C ABI).
#pragma once
#include "common.cuh"

namespace gato {
// out[b] = coef * L(psi[b]) + V * psi[b]; dot_dev[b] = dv * <psi[b], out[b]>.
int stencil_apply(int dtype, const void* psi, const void* V, void* out, int nb, int nx, int ny,
                  int nz, int64_t bstride, double coef, int boundary, int order, double* dot_dev,
                  double dv, cudaStream_t s);
}  // namespace gato
