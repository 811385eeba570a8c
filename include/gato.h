/*
 * gato.h -- C ABI of libgato_cuda, the GB300 (sm_103a) implementation of
 * GATO's Fock-operator path.
 *
 * Conventions
 * -----------
 * - Every function returns GATO_OK (0) or a negative status; the message of
 *   the last failure on the calling thread is available from gato_last_error.
 * - Array arguments are raw DEVICE pointers owned by the caller and never
 *   freed by the library. Fields are C-order (nx, ny, nz) with z fastest,
 *   the reference's `indexing="ij"` layout. A block of n fields is stored
 *   field-major: n consecutive N^3 arrays (the reference's (N,N,N,n)
 *   orbital arrays are the transposed view of this).
 * - dtype selects the arithmetic of the field kernels: GATO_F64 (the plain
 *   FP64 path) or GATO_F32 (the mixed path: FP32 fields, stencils and FFTs,
 *   with FP64/float-float accumulation for every reduction and FP64 for the
 *   tridiagonal eigensolve and Lanczos coefficients).
 * - Scalar results (energies, dot products, eigenvalues) are written to
 *   caller-provided DEVICE doubles so nothing forces a host synchronisation.
 * - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * - Plans and operators allocate their workspace once, at creation; their
 *   apply calls allocate nothing. A plan or operator is used from one stream
 *   at a time.
 *
 * Each entry point cites the reference function it replaces, by path inside
 * the ezequielgarcia/gato source tree (src/gato/...).
 */
#ifndef GATO_H
#define GATO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum gato_status {
    GATO_OK = 0,
    GATO_EBADARG = -1,      /* the reference raises ValueError            */
    GATO_ECUDA = -2,        /* a CUDA runtime/driver call failed          */
    GATO_ETIMEOUT = -3,     /* a bounded device wait expired              */
    GATO_ENOMEM = -4,       /* device allocation failed                   */
    GATO_EUNSUPPORTED = -5, /* the reference raises NotImplementedError   */
    GATO_EKEY = -6          /* the reference raises KeyError              */
};

enum gato_dtype { GATO_F64 = 0, GATO_F32 = 1 };
enum gato_boundary { GATO_DIRICHLET = 0, GATO_PERIODIC = 1 };

typedef struct gato_poisson_plan* gato_poisson_t;
typedef struct gato_nonlocal* gato_nonlocal_t;
typedef struct gato_operator* gato_op_t;

/* ---- library ------------------------------------------------------------
 * Library services with no reference counterpart (the reference is Python
 * and reports errors as exceptions, which the Python layer raises from the
 * status and this message).                                                */
int gato_version(void);
int gato_last_error(char* buf, size_t len);
/* Reads and clears the device error word set by bounded spin-waits. */
int gato_device_status(int* status_out, void* stream);
/* Kernel launches issued by this library since it was loaded (all threads). */
long long gato_launch_count(void);

/* ---- grid.py: integrate / inner_product / norm_sq / normalize ----------
 * grid.py:57-73. out_dev[0] = scale * sum_i a_i * b_i  (b == NULL: sum_i a_i).
 * The FP32 path accumulates products in float-float and blocks in FP64.   */
int gato_dot(int dtype, const void* a, const void* b, int64_t n, double scale,
             double* out_dev, void* stream);
/* gato_dot for callers that cannot allocate device memory: hosts that own
 * all device memory through their own allocator and forbid the CUDA
 * runtime's, and latency-critical threads that must not block in cudaMalloc.
 * No counterpart in the reference. Its partial sums live in a library-owned
 * static device array (512 KiB per GPU, resident until exit) instead of
 * lazily allocated scratch; the first call on a device looks up that array's
 * address and caches it. n is limited to 2^27
 * elements (GATO_EBADARG beyond). Calls share the array: any two calls whose
 * kernels can run at the same time on the GPU race.                      */
int gato_dot_noalloc(int dtype, const void* a, const void* b, int64_t n, double scale,
                     double* out_dev, void* stream);
/* a[i] *= 1/sqrt(norm_dev[0]) -- the divide of grid.py:72-73.            */
int gato_normalize(int dtype, void* a, int64_t n, const double* norm_sq_dev, void* stream);

/* ---- operators.py: laplacian / kinetic; hamiltonian.py: apply ----------
 * operators.py:40-130, hamiltonian.py:25-35.
 * out[b] = lap_coef * L(psi[b]) + V * psi[b] for b < nb, where L is the
 * 7-point (order 2) or 13-point (order 4) stencil sum without the 1/h^2
 * (lap_coef carries it: 1/h^2 for laplacian, -0.5/h^2 for kinetic). V may
 * be NULL. If dot_dev != NULL, dot_dev[b] = dv * <psi[b], out[b]> (the
 * expectation of hamiltonian.py:29-31). Bad order/boundary: GATO_EBADARG,
 * as operators.py:64,80-83 raise ValueError.                             */
int gato_stencil_apply(int dtype, const void* psi, const void* V, void* out, int nb,
                       int nx, int ny, int nz, double lap_coef, int boundary, int order,
                       double* dot_dev, double dv, void* stream);
/* Tile shape of the stencil's TMA kernel: rows per thread 4 (128-thread
 * CTAs) or 2 (256-thread CTAs), 0 = default. Process-wide; chosen by the
 * autotuner. No reference counterpart (a tuning knob of this library).   */
int gato_stencil_tune(int rows_per_thread);

/* ---- potentials.py / pseudopotentials.py --------------------------------
 * V = -sum_k Z_k / sqrt(|r-R_k|^2 + eps^2): potentials.py:16-61.
 * pos_host: K*3 doubles (host), Z_host: K doubles (host).               */
int gato_softened_coulomb(int dtype, void* V, int N, double L, int K, const double* pos_host,
                          const double* Z_host, double eps, void* stream);
/* HGH local part, pseudopotentials.py:201-253. c_host: K*4 doubles.       */
int gato_hgh_local(int dtype, void* V, int N, double L, int K, const double* pos_host,
                   const double* Zion_host, const double* rloc_host, const double* c_host,
                   void* stream);
/* Separable non-local part, pseudopotentials.py:265-383. Channels are
 * listed atom by atom: atom k owns nch_host[k] channels; channel c has
 * angular momentum ell_host[c] (<= 2 else GATO_EUNSUPPORTED), width
 * r_host[c], n_host[c] <= 3 radial projectors and the symmetric matrix
 * h_host[9c .. 9c+8] (row-major 3x3, upper-left n x n used). Projectors
 * are evaluated on per-atom boxes of radius cut_sigmas * max r_l (the
 * Gaussian tail beyond is below 1e-16 relative at cut_sigmas = 8.6).      */
int gato_nonlocal_create(int dtype, int N, double L, int K, const double* pos_host,
                         const int* nch_host, const int* ell_host, const double* r_host,
                         const int* n_host, const double* h_host, double cut_sigmas,
                         gato_nonlocal_t* out);
/* Frees the projector set (no reference counterpart: the reference
 * rebuilds the projector fields on every apply).                          */
int gato_nonlocal_destroy(gato_nonlocal_t nl);
/* out[b] += V_nl psi[b] for b < nb: hgh_nonlocal_apply (pseudopotentials.py:360-383). */
int gato_nonlocal_apply(gato_nonlocal_t nl, const void* psi, void* out, int nb, void* stream);
/* energy_dev[0] = 2 * sum_b <psi_b | V_nl | psi_b> (scf.py:217-221).     */
int gato_nonlocal_energy(gato_nonlocal_t nl, const void* psi, int nb, double* energy_dev, void* stream);

/* ---- solvers/poisson.py --------------------------------------------------
 * Plan = Hockney doubled grid M = 2N with the transform of the softened
 * kernel (poisson.py:29-44) computed once, in FP64, and kept as the
 * (M/2+1)^3 octant of its even spectrum. max_fields bounds how many
 * complex fields (two real densities each) one batched launch holds.
 * M must factor into 2, 3, 5, 7 (else GATO_EUNSUPPORTED).               */
int gato_poisson_create(int dtype, int N, double h, double eps, int max_fields,
                        gato_poisson_t* out, void* stream);
int gato_poisson_destroy(gato_poisson_t plan);
/* J = hartree_potential(rho): poisson.py:47-79.                           */
int gato_hartree_potential(gato_poisson_t plan, const void* rho, void* J, void* stream);
/* E_dev[0] = 0.5 * dV * sum rho J[rho]: poisson.py:82-92. FP64 plans on the
 * register engine evaluate it from the spectrum, 0.5 * dV * sum_k ghat |rho^|^2
 * (Parseval on the doubled grid, equal in exact arithmetic), without the
 * inverse transforms.                                                      */
int gato_hartree_energy(gato_poisson_t plan, const void* rho, double* E_dev, void* stream);
/* Profiling hook (no reference counterpart): runs stage 1 (y forward),
 * 2 (x forward, kernel multiply, x inverse) or 3 (y inverse) of the pair-
 * solve pipeline alone on nf fields of the plan's own buffers.           */
int gato_poisson_stage(gato_poisson_t plan, int stage, int nf, void* stream);
/* Tuning (no reference counterpart): fields per launch group (0 = all of
 * max_fields) and FFT engine (0: register-resident two-pass kernels for
 * M in {32,48,64,80,96,128,160,192,256,320}, with the multi-field z
 * forward for two or more fields; 1: generic Stockham; 2: the register
 * kernels with one z-forward CTA per field; 3: the multi-field z forward
 * from three fields; 4: as 0 with the scalar FP32 column passes instead of
 * the packed two-line ones, which FP32 plans use for M in
 * {128,160,192,256,320}, and a z forward that stages once per CTA
 * instead of persistent CTAs with double-buffered staging).              */
int gato_poisson_tune(gato_poisson_t plan, int group, int engine);

/* ---- scf.py ----------------------------------------------------------------
 * rho = 2 sum_i phi_i^2 (scf.py:61-63), orbitals field-major.             */
int gato_density(int dtype, const void* orbitals, int n, int64_t npts, void* rho, void* stream);
/* rho = a * rho_new + (1 - a) * rho (scf.py:422-423).                      */
int gato_mix(int dtype, void* rho, const void* rho_new, int64_t npts, double a, void* stream);
/* out = a x + b y: the Hamiltonian's V_ext + V_H (scf.py:399-409) and any
 * elementwise combination the SCF loop needs.                            */
int gato_axpby(int dtype, const void* x, const void* y, void* out, int64_t npts, double a, double b,
               void* stream);
/* dst = (dst dtype) src, n elements: the precision changes between the FP32
 * Fock applies and the FP64 density / Hartree / energy of the mixed SCF.
 * No reference counterpart: the reference computes in FP64 throughout.     */
int gato_convert(int src_dtype, const void* src, int dst_dtype, void* dst, int64_t n, void* stream);
/* out_dev[0] = scale * sum_i a_i w_i b_i: <psi|V|psi> of potential_energy
 * (observables.py:26-30).                                                  */
int gato_dot_weighted(int dtype, const void* a, const void* w, const void* b, int64_t n, double scale,
                      double* out_dev, void* stream);
/* out = sum_k fields[k]: the Lanczos seed sum(orbitals, axis=-1) (scf.py:417). */
int gato_field_sum(int dtype, const void* fields, int nf, int64_t npts, void* out, void* stream);
/* out += coef * K psi, K psi = sum_j phi_j J[phi_j psi]: scf.py:66-85.     */
int gato_exchange_apply(gato_poisson_t plan, const void* psi, const void* orbitals, int n_orb,
                        void* out, double coef, void* stream);

/* Operator: F psi = -1/2 L psi + V psi [+ V_nl psi] [- K psi], the matrix-
 * free map of hamiltonian.py:25-27 (no nonlocal, no orbitals) and
 * scf.py:88-111 / 114-158 (RHFFock with V = V_ext + V_H). Pointers are
 * borrowed; the operator may be re-pointed between calls.               */
int gato_op_create(int dtype, int N, double h, int order, int boundary, gato_op_t* out);
int gato_op_destroy(gato_op_t op);
int gato_op_set_potential(gato_op_t op, const void* V);
int gato_op_set_nonlocal(gato_op_t op, gato_nonlocal_t nl);
int gato_op_set_exchange(gato_op_t op, gato_poisson_t plan, const void* orbitals, int n_orb);
/* Tuning (no reference counterpart): 1 (default) runs the stencil and the
 * non-local projectors of an apply on the operator's own side stream,
 * concurrently with the exchange's FFT passes, joined before the first
 * kernel that accumulates into the outputs; 0 runs everything on the
 * caller's stream in order. Either way the call is ordered on the caller's
 * stream like any other launch.                                          */
int gato_op_overlap(gato_op_t op, int on);
/* Block-apply epilogue: 0 = auto, 1 = J_ij fields then one pair pass, 2 =
 * accumulate every output in the z-inverse epilogue. No reference
 * counterpart (a tuning knob of this library, set by the autotuner).      */
int gato_op_tune(gato_op_t op, int block_epilogue);
/* out = F in, one vector.                                                  */
int gato_op_apply(gato_op_t op, const void* in, void* out, void* stream);
/* out_i = F phi_i for the operator's own n_orb orbitals, with the
 * n(n+1)/2 pair potentials J[phi_i phi_j] each used for both i and j.    */
int gato_op_apply_block(gato_op_t op, void* out, void* stream);
/* terms_dev[0..4] = (kinetic, v_ext, v_nl, hartree, exchange) of
 * decompose_rhf_energy (scf.py:194-265) for the operator's orbitals,
 * with v_ext taken against V_ext_dev (the operator's V may hold V_H).
 * Hartree and exchange come from one batched pass over the density and the
 * pair densities; FP64 operators take it in the spectral form of
 * gato_hartree_energy.                                                    */
int gato_op_energy_terms(gato_op_t op, const void* V_ext, double* terms_dev, void* stream);

/* ---- solvers/lanczos.py ----------------------------------------------------
 * lanczos (lanczos.py:110-206): m steps from psi0 with full reorthogonal-
 * isation (classical Gram-Schmidt, reorth_passes passes, coefficients in
 * FP64), tridiagonal eigensolve on the device (bisection + inverse
 * iteration, FP64), Ritz vectors of the K lowest pairs written field-major
 * to evecs (K x N^3). krylov: (m+1) x N^3 workspace. evals_dev: K doubles;
 * alphas_dev/betas_dev: m doubles each; flag_dev[0] = any beta_j < tol for
 * j < max(m-1, 1) (the `converged` of lanczos.py:199). Eigenvector signs
 * are fixed so that each Ritz vector's largest tridiagonal component is
 * positive (LAPACK leaves the sign arbitrary).                          */
int gato_lanczos(gato_op_t op, const void* psi0, int m, int K, double tol, int reorth_passes,
                 void* krylov, double* evals_dev, void* evecs, double* alphas_dev,
                 double* betas_dev, int* flag_dev, void* stream);
/* Tuning (no reference counterpart): basis sweeps per step of the FP32
 * Lanczos loop: 1 = one sweep (the operator applied to the unorthogonalised
 * three-term vector, its image recovered from the Lanczos relation; used
 * where m <= 200 and n is a multiple of 128), 2 = the classical Gram-Schmidt
 * coefficient and correction sweeps. Default 1.                          */
int gato_lanczos_tune(int sweeps);
/* The same algorithm in three pieces, for a matvec the caller supplies (the
 * duck-typed `H.apply` of lanczos.py:110-170): begin writes v_0 into slot 0;
 * the caller writes F v_j into slot j+1 and calls step(j), which
 * reorthogonalises and normalises it in place and records alpha_j, beta_j;
 * finish solves the tridiagonal problem and forms the Ritz vectors.       */
int gato_lanczos_begin(int dtype, int64_t n, double dV, const void* psi0, void* krylov, int m,
                       int K, void* stream);
int gato_lanczos_step(int dtype, int64_t n, double dV, void* krylov, int j, int m, int K,
                      int reorth_passes, double* alphas_dev, double* betas_dev, void* stream);
int gato_lanczos_finish(int dtype, int64_t n, const void* krylov, int m, int K, double tol,
                        const double* alphas_dev, const double* betas_dev, double* evals_dev,
                        void* evecs, int* flag_dev, void* stream);

/* ---- solvers/imag_time.py:29-65, observables.py:41-59 ----------------------
 * gato_imag_time: psi (in/out, N^3) <- n_steps Euler steps of
 * psi <- (psi - dt H psi) / |psi - dt H psi| with H = -1/2 Laplacian + V
 * (V null: no potential), after normalising psi. energies_dev receives the
 * Rayleigh quotient after every step i with i % log_every == 0 or
 * i == n_steps - 1, in order. The step is replayed as a CUDA graph.
 * gato_radial_density: hist_dev[k] = sum over grid points with radius in
 * [edges[k], edges[k+1]) (last bin closed) of (re^2 + im^2) dV, im optional;
 * edges_host holds n_bins + 1 increasing radii (numpy.histogram binning).  */
int gato_imag_time(int dtype, void* psi, const void* V, int N, double h, int order, int boundary, double dt,
                   int n_steps, int log_every, double* energies_dev, void* stream);
int gato_radial_density(int dtype, const void* re, const void* im, int N, double L, const double* edges_host,
                        int n_bins, double* hist_dev, void* stream);

/* ---- physics/water.py: Hellmann-Feynman forces -----------------------------
 * grad_host (K*3, host doubles, ACCUMULATED into) += d/dR of the R-dependent
 * energy at fixed orbitals: int rho V_loc(R) (pseudopotentials.py:201-253)
 * and 2 sum_i <phi_i|V_nl(R)|phi_i> (pseudopotentials.py:330-383); the
 * reference obtains these with jax.grad (water.py:221-241).              */
int gato_hgh_local_grad(int dtype, const void* rho, int N, double L, int K, const double* pos_host,
                        const double* Zion_host, const double* rloc_host, const double* c_host,
                        double* grad_host, void* stream);
/* The projector term alone: 2 sum_i <phi_i|V_nl(R)|phi_i> differentiated
 * in R (pseudopotentials.py:330-383 under water.py:221-241's jax.grad).   */
int gato_nonlocal_grad(gato_nonlocal_t nl, const void* orbitals, int n, double* grad_host, void* stream);
/* grad_host (K*3) += d/dR of int rho V_ext for the multi-centre softened
 * Coulomb V_ext = -sum_k Z_k / sqrt(|r - R_k|^2 + eps^2) (potentials.py:39-61);
 * the H2 driver's force, which the reference takes with jax.grad
 * (physics/h2.py:109-135).                                                 */
int gato_softened_coulomb_grad(int dtype, const void* rho, int N, double L, int K,
                               const double* pos_host, const double* Z_host, double eps,
                               double* grad_host, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GATO_H */
