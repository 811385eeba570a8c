// The Fock / Hamiltonian operator of hamiltonian.py:25-35 and scf.py:88-158,
// and the RHF energy decomposition of scf.py:194-265.
//
// apply      : stencil(+V) writes out; V_nl scatter-adds; the exchange pass
//              subtracts sum_j phi_j J[phi_j psi] in its final z-row epilogue.
//              The stencil and V_nl run on the operator's side stream beside
//              the exchange's transforms and join before the epilogue (in the
//              block apply: before the pair pass).
// apply_block: F phi_i for every occupied orbital with the n(n+1)/2 pair
//              potentials J[phi_i phi_j], each feeding both phi_i and phi_j:
//              either the pipeline writes the J_ij fields and one elementwise
//              pass subtracts sum_j phi_j J_ij from every output (each J read
//              once), or the z-inverse epilogue accumulates every output in
//              registers (no J fields); gato_op_tune picks, the autotuner times both.
// energy     : kinetic via the stencil's fused <phi, T phi> reduction (no
//              store), V_ext and V_nl by reductions, E_H and E_x from one
//              batched pair-solve pass in energy mode (rho with weight 1/2,
//              pairs with -1 (i = j) or -2 (i < j)); FP64 plans stop that pass
//              at the x-forward spectrum (Parseval).
#include "op.cuh"
#include "stencil.cuh"

namespace gato {

int exchange_args(PassArgs& a, const void* psi, const void* orbitals, int n_orb, size_t esz,
                  int64_t n3, void* out, double coef);

namespace {

template <typename T>
__global__ void k_vext_energy(const T* __restrict__ orb, int n, const T* __restrict__ V, int64_t npts,
                              double* part) {
  __shared__ double sh[32];
  Acc<T> acc;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T v = V[i];
    for (int k = 0; k < n; ++k) {
      const T p = orb[(int64_t)k * npts + i];
      acc.add_prod(p * v, p);
    }
  }
  const double s = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_sum_scaled(const double* in, int n, double scale, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += in[i];
    out[0] = scale * s;
  }
}

}  // namespace

// The operator's side stream and its fork/join events, created on first use.
static int op_side(gato_operator& op) {
  if (op.side) return GATO_OK;
  GATO_CUDA_TRY(cudaStreamCreateWithFlags(&op.side, cudaStreamNonBlocking));
  GATO_CUDA_TRY(cudaEventCreateWithFlags(&op.ev_fork, cudaEventDisableTiming));
  GATO_CUDA_TRY(cudaEventCreateWithFlags(&op.ev_join, cudaEventDisableTiming));
  return GATO_OK;
}

// out[b] = (-1/2 L + V) psi[b] (+ V_nl psi[b]) for nb fields, on stream ls.
static int local_part(gato_operator& op, const void* in, void* out, int nb, cudaStream_t ls) {
  const double coef = -0.5 / (op.h * op.h);
  GATO_TRY(stencil_apply(op.dtype, in, op.V, out, nb, op.N, op.N, op.N, op_n3(op), coef, op.boundary,
                         op.order, nullptr, op.dV, ls));
  if (op.nl) GATO_TRY(nonlocal_apply(op.nl->n, in, out, nb, ls));
  return GATO_OK;
}

// Runs the local part on the side stream from this point of s; returns the join event
// (null when the local part ran on s itself).
static int fork_local(gato_operator& op, const void* in, void* out, int nb, cudaStream_t s,
                      cudaEvent_t* join) {
  *join = nullptr;
  if (!op.overlap) return local_part(op, in, out, nb, s);
  GATO_TRY(op_side(op));
  GATO_CUDA_TRY(cudaEventRecord(op.ev_fork, s));
  GATO_CUDA_TRY(cudaStreamWaitEvent(op.side, op.ev_fork, 0));
  GATO_TRY(local_part(op, in, out, nb, op.side));
  GATO_CUDA_TRY(cudaEventRecord(op.ev_join, op.side));
  *join = op.ev_join;
  return GATO_OK;
}

int op_apply(gato_operator& op, const void* in, void* out, cudaStream_t s) {
  if (op.n_orb <= 0) return local_part(op, in, out, 1, s);
  cudaEvent_t join = nullptr;
  GATO_TRY(fork_local(op, in, out, 1, s, &join));
  PassArgs a;
  GATO_TRY(exchange_args(a, in, op.orbitals, op.n_orb, op_esize(op), op_n3(op), out, -1.0));
  return poisson_run(op.pp->p, a, EPI_ACC, true, nullptr, s, join);
}

static void block_pairs(PassArgs& a, const gato_operator& op, void* out, bool energy) {
  const int n = op.n_orb;
  const size_t es = op_esize(op);
  const int64_t n3 = op_n3(op);
  for (int j = 0; j < n; ++j) {
    a.in[j] = (const char*)op.orbitals + (size_t)j * n3 * es;
    if (!energy) a.out[j] = (char*)out + (size_t)j * n3 * es;
  }
  a.nout = energy ? 0 : n;
  int part = 0;
  const int nd = n, no = n * (n - 1) / 2;
  const int f_mixed = (1 + nd + no + 1) / 2, f_split = 1 + (nd + 1) / 2 + (no + 1) / 2;
  if (energy && op.pp && poisson_fe_supported(op.pp->p) && f_split < 2 * f_mixed) {
    // The spectral energy pass (half the work of a field's full solve) sums
    // both parts of a field with one weight: the density rides alone, the
    // diagonal pairs (weight -1) and the off-diagonal pairs (weight -2) fill
    // fields of their own.
    a.in[n] = op.rho;
    PartDesc& d = a.f[0].p[0];
    d.a = (int8_t)n;
    d.ew = 0.5;
    d.eslot = 0;
    int nf = 1;
    for (int w = 0; w < 2; ++w) {
      part = 0;
      for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
          if ((i == j) != (w == 0)) continue;
          PartDesc& e = a.f[nf + part / 2].p[part % 2];
          e.a = (int8_t)i;
          e.b = (int8_t)j;
          e.ew = i == j ? -1.0 : -2.0;   // E_x = -sum_ij <phi_i phi_j | J[phi_i phi_j]>
          e.eslot = 1;
          ++part;
        }
      nf += (part + 1) / 2;
    }
    a.nf = nf;
    return;
  }
  if (energy) {
    // the density rides first: E_H = 1/2 dV sum rho J[rho]
    a.in[n] = op.rho;
    PartDesc& d = a.f[0].p[0];
    d.a = (int8_t)n;
    d.ew = 0.5;
    d.eslot = 0;
    part = 1;
  }
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j, ++part) {
      PartDesc& d = a.f[part / 2].p[part % 2];
      d.a = (int8_t)i;
      d.b = (int8_t)j;
      if (energy) {
        d.ew = i == j ? -1.0 : -2.0;   // E_x = -sum_ij <phi_i phi_j | J[phi_i phi_j]>
        d.eslot = 1;
      } else {
        d.nt = i == j ? 1 : 2;
        d.to[0] = (int8_t)i;
        d.tc[0] = (int8_t)j;
        d.coef[0] = -1.f;
        d.to[1] = (int8_t)j;
        d.tc[1] = (int8_t)i;
        d.coef[1] = -1.f;
      }
    }
  a.nf = (part + 1) / 2;
}

}  // namespace gato

using namespace gato;

extern "C" int gato_op_create(int dtype, int N, double h, int order, int boundary, gato_op_t* out) {
  if (!out) return fail(GATO_EBADARG, "gato_op_create: out is NULL");
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  if (order != 2 && order != 4) return fail(GATO_EBADARG, "Unknown order %d; expected 2 or 4.", order);
  if (boundary != GATO_DIRICHLET && boundary != GATO_PERIODIC)
    return fail(GATO_EBADARG, "Unknown boundary %d; expected 'dirichlet' or 'periodic'.", boundary);
  if (N < 1 || h <= 0) return fail(GATO_EBADARG, "gato_op_create: bad grid");
  auto* op = new gato_operator();
  op->dtype = dtype;
  op->N = N;
  op->h = h;
  op->dV = h * h * h;
  op->order = order;
  op->boundary = boundary;
  if (cudaMalloc(&op->dscratch, 64 * sizeof(double)) != cudaSuccess) {
    delete op;
    return fail(GATO_ENOMEM, "gato_op_create: allocation failed");
  }
  *out = op;
  return GATO_OK;
}

extern "C" int gato_op_destroy(gato_op_t op) {
  if (!op) return GATO_OK;
  free_after_pending({op->dscratch, op->rho, op->jbuf});   // waits for the device first
  if (op->side) {
    cudaStreamSynchronize(op->side);
    cudaStreamDestroy(op->side);
    cudaEventDestroy(op->ev_fork);
    cudaEventDestroy(op->ev_join);
  }
  delete op;
  return GATO_OK;
}

extern "C" int gato_op_set_potential(gato_op_t op, const void* V) {
  if (!op) return fail(GATO_EBADARG, "null operator");
  op->V = V;
  return GATO_OK;
}

extern "C" int gato_op_set_nonlocal(gato_op_t op, gato_nonlocal_t nl) {
  if (!op) return fail(GATO_EBADARG, "null operator");
  if (nl && (nl->n.dtype != op->dtype || nl->n.N != op->N))
    return fail(GATO_EBADARG, "nonlocal set does not match the operator's dtype/grid");
  op->nl = nl;
  return GATO_OK;
}

extern "C" int gato_op_set_exchange(gato_op_t op, gato_poisson_t plan, const void* orbitals,
                                    int n_orb) {
  if (!op) return fail(GATO_EBADARG, "null operator");
  if (n_orb > 0 && (!plan || !orbitals)) return fail(GATO_EBADARG, "exchange needs a plan and orbitals");
  if (plan && (plan->p.dtype != op->dtype || plan->p.N != op->N))
    return fail(GATO_EBADARG, "poisson plan does not match the operator's dtype/grid");
  if (n_orb > kMaxIn - 2) return fail(GATO_EUNSUPPORTED, "at most %d orbitals", kMaxIn - 2);
  op->pp = plan;
  op->orbitals = orbitals;
  op->n_orb = n_orb;
  return GATO_OK;
}

extern "C" int gato_op_apply(gato_op_t op, const void* in, void* out, void* stream) {
  if (!op || !in || !out) return fail(GATO_EBADARG, "gato_op_apply: bad arguments");
  return op_apply(*op, in, out, as_stream(stream));
}

extern "C" int gato_op_apply_block(gato_op_t op, void* out, void* stream) {
  if (!op || !out || op->n_orb < 1) return fail(GATO_EBADARG, "gato_op_apply_block: needs orbitals");
  if (op->n_orb > kMaxOut) return fail(GATO_EUNSUPPORTED, "block apply: at most %d orbitals", kMaxOut);
  cudaStream_t s = as_stream(stream);
  cudaEvent_t join = nullptr;
  GATO_TRY(fork_local(*op, op->orbitals, out, op->n_orb, s, &join));
  PassArgs a;
  block_pairs(a, *op, out, false);
  if (op->block_epi != 2 && poisson_j_supported(op->pp->p)) {
    // pair potentials to J fields, then one elementwise pass: out_i -= sum_j phi_j J_ij
    const size_t need = (size_t)2 * a.nf * op_n3(*op) * op_esize(*op);
    if (op->jbuf_bytes < need) {
      free_after_pending({op->jbuf});
      op->jbuf = nullptr;
      op->jbuf_bytes = 0;
      GATO_CUDA_TRY(cudaMalloc(&op->jbuf, need));
      op->jbuf_bytes = need;
    }
    a.jbase = op->jbuf;
    a.jstride = op_n3(*op);
    GATO_TRY(poisson_run(op->pp->p, a, EPI_J, false, nullptr, s));
    if (join) GATO_CUDA_TRY(cudaStreamWaitEvent(s, join, 0));
    return pair_exchange(op->dtype, op->orbitals, op->n_orb, op->jbuf, out, op_n3(*op), s);
  }
  return poisson_run(op->pp->p, a, EPI_ACC, true, nullptr, s, join);
}

extern "C" int gato_op_overlap(gato_op_t op, int on) {
  if (!op || (on != 0 && on != 1)) return fail(GATO_EBADARG, "gato_op_overlap: on must be 0 or 1");
  op->overlap = on;
  return GATO_OK;
}

extern "C" int gato_op_tune(gato_op_t op, int block_epilogue) {
  if (!op || block_epilogue < 0 || block_epilogue > 2)
    return fail(GATO_EBADARG, "gato_op_tune: block epilogue must be 0, 1 or 2");
  op->block_epi = block_epilogue;
  return GATO_OK;
}

extern "C" int gato_op_energy_terms(gato_op_t op, const void* V_ext, double* terms, void* stream) {
  if (!op || !terms || op->n_orb < 1) return fail(GATO_EBADARG, "gato_op_energy_terms: needs orbitals");
  cudaStream_t s = as_stream(stream);
  const int n = op->n_orb;
  const int64_t n3 = op_n3(*op);
  double* ds = op->dscratch;   // [0..15] per-orbital kinetic, [16..] misc
  // kinetic: 2 sum_i <phi_i | T phi_i>, reduced inside the stencil (no store)
  const double coef = -0.5 / (op->h * op->h);
  if (n > 16) return fail(GATO_EUNSUPPORTED, "energy terms: at most 16 orbitals");
  GATO_TRY(stencil_apply(op->dtype, op->orbitals, nullptr, nullptr, n, op->N, op->N, op->N, n3, coef,
                         op->boundary, op->order, ds, op->dV, s));
  k_sum_scaled<<<1, 32, 0, s>>>(ds, n, 2.0, terms + 0);
  GATO_LAUNCH_TRY();
  // v_ext: 2 sum_i <phi_i | V_ext phi_i>
  if (V_ext) {
    double* part = (double*)stream_scratch(s, kRedBlocks * sizeof(double));
    if (!part) return fail(GATO_ENOMEM, "scratch");
    const unsigned nb = grid_for(n3, 256, kRedBlocks);
    if (op->dtype == GATO_F64)
      k_vext_energy<double><<<nb, 256, 0, s>>>((const double*)op->orbitals, n, (const double*)V_ext, n3, part);
    else
      k_vext_energy<float><<<nb, 256, 0, s>>>((const float*)op->orbitals, n, (const float*)V_ext, n3, part);
    GATO_LAUNCH_TRY();
    GATO_TRY(finalize_sums(part, 1, nb, 2.0 * op->dV, terms + 1, s));
  } else {
    GATO_CUDA_TRY(cudaMemsetAsync(terms + 1, 0, sizeof(double), s));
  }
  // v_nl
  if (op->nl) GATO_TRY(nonlocal_energy(op->nl->n, op->orbitals, n, terms + 2, s));
  else GATO_CUDA_TRY(cudaMemsetAsync(terms + 2, 0, sizeof(double), s));
  // hartree + exchange
  if (!op->pp) return fail(GATO_EBADARG, "energy terms need a Poisson plan");
  if (!op->rho) GATO_CUDA_TRY(cudaMalloc(&op->rho, n3 * op_esize(*op)));
  GATO_TRY(gato_density(op->dtype, op->orbitals, n, n3, op->rho, s));
  PassArgs a;
  block_pairs(a, *op, nullptr, true);
  return poisson_run(op->pp->p, a, EPI_ENERGY, false, terms + 3, s);
}
