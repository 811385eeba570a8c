// Matrix-free operator F = -1/2 L + V [+ V_nl] [- K] (internal API).
#pragma once
#include "common.cuh"
#include "hgh.cuh"
#include "poisson.cuh"

struct gato_operator {
  int dtype = GATO_F64;
  int N = 0;
  double h = 0, dV = 0;
  int order = 4, boundary = GATO_DIRICHLET;
  const void* V = nullptr;
  gato_nonlocal* nl = nullptr;
  gato_poisson_plan* pp = nullptr;
  const void* orbitals = nullptr;
  int n_orb = 0;
  double* dscratch = nullptr;   // small device doubles
  void* rho = nullptr;          // N^3 density scratch for the energy terms
  void* jbuf = nullptr;         // pair potentials J_ij of the block apply
  size_t jbuf_bytes = 0;
  int block_epi = 0;            // block apply epilogue: 0 auto, 1 J fields + pair pass, 2 fused
  // The local part (stencil + V, non-local projectors) runs on a side stream beside the exchange's
  // transforms and joins before the first kernel that touches the outputs again.
  int overlap = 1;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace gato {
int op_apply(gato_operator& op, const void* in, void* out, cudaStream_t s);
inline size_t op_esize(const gato_operator& op) { return op.dtype == GATO_F64 ? 8 : 4; }
inline int64_t op_n3(const gato_operator& op) { return (int64_t)op.N * op.N * op.N; }
}  // namespace gato
