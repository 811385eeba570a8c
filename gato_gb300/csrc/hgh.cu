// HGH pseudopotentials and softened Coulomb potentials on the grid
// (pseudopotentials.py:201-405, potentials.py:16-61), plus the analytic
// position derivatives the Hellmann-Feynman forces need (the reference takes
// them with jax.grad, physics/water.py:221-241).
//
// The non-local projectors are Gaussians; each atom's projectors are
// evaluated once per geometry on a box of radius cut_sigmas * max r_l around
// it (the reference rebuilds full-grid fields on every apply). An apply is
// one launch of a thread-block cluster per vector: its CTAs split the box
// points, reduce the overlaps <p_q|psi> through distributed shared memory,
// form the h-matrix contraction and scatter-add each atom's projectors in
// turn (a cluster barrier between atoms, so overlapping boxes never race).
#include <cmath>
#include <vector>

#include <cooperative_groups.h>

#include "hgh.cuh"

namespace gato {

namespace {

constexpr int kMaxAtoms = 32;

struct AtomTable {
  int K;
  double x[kMaxAtoms], y[kMaxAtoms], z[kMaxAtoms];
  double Z[kMaxAtoms], rloc[kMaxAtoms], c[kMaxAtoms][4];
};

__device__ __forceinline__ double axis_coord(int i, double L, double h) {
  return -L / 2 + (i + 0.5) * h;  // grid.py:44
}

template <typename T>
__global__ void k_softened(T* V, int N, double L, double h, AtomTable at, double eps) {
  const int64_t n3 = (int64_t)N * N * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % N), y = (int)((i / N) % N), x = (int)(i / ((int64_t)N * N));
    const double X = axis_coord(x, L, h), Y = axis_coord(y, L, h), Zc = axis_coord(z, L, h);
    double v = 0.0;
    for (int k = 0; k < at.K; ++k) {
      const double dx = X - at.x[k], dy = Y - at.y[k], dz = Zc - at.z[k];
      v += -at.Z[k] / sqrt(dx * dx + dy * dy + dz * dz + eps * eps);
    }
    V[i] = (T)v;
  }
}

// V_loc of one centre at distance r (pseudopotentials.py:214-227).
__device__ __forceinline__ double hgh_vloc(double r, double Z, double rloc, const double* c) {
  const double rho = r / rloc;
  const double erf_term = -Z * erf(r / (1.4142135623730951 * rloc)) / r;
  const double rho2 = rho * rho;
  const double poly = c[0] + c[1] * rho2 + c[2] * rho2 * rho2 + c[3] * rho2 * rho2 * rho2;
  return erf_term + exp(-0.5 * rho2) * poly;
}

template <typename T>
__global__ void k_hgh_local(T* V, int N, double L, double h, AtomTable at) {
  const int64_t n3 = (int64_t)N * N * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % N), y = (int)((i / N) % N), x = (int)(i / ((int64_t)N * N));
    const double X = axis_coord(x, L, h), Y = axis_coord(y, L, h), Zc = axis_coord(z, L, h);
    double v = 0.0;
    for (int k = 0; k < at.K; ++k) {
      const double dx = X - at.x[k], dy = Y - at.y[k], dz = Zc - at.z[k];
      const double r = sqrt(dx * dx + dy * dy + dz * dz + 1e-30);
      v += hgh_vloc(r, at.Z[k], at.rloc[k], at.c[k]);
    }
    V[i] = (T)v;
  }
}

// dV_loc/dr of one centre. For r/(sqrt2 r_loc) < 1e-3 the erf part uses its
// Taylor series, which avoids the cancellation of erf'(u)/r - erf(u)/r^2.
template <typename R>
__device__ __forceinline__ R hgh_dvloc_dr(R r, R Z, R rloc, const double* c) {
  const R a = (R)1.4142135623730951 * rloc;
  const R u = r / a;
  const R two_sqrtpi = (R)1.1283791670955126;
  R f;
  if (u < (R)1e-3) {
    f = two_sqrtpi * ((R)(-2.0 / 3.0) * u + (R)0.4 * u * u * u) / (a * a);
  } else {
    f = two_sqrtpi * exp(-u * u) / (a * r) - erf(u) / (r * r);
  }
  const R d_erf = -Z * f;
  const R rho2 = (r / rloc) * (r / rloc);
  const R poly = (R)c[0] + (R)c[1] * rho2 + (R)c[2] * rho2 * rho2 + (R)c[3] * rho2 * rho2 * rho2;
  const R dpoly = (R)c[1] + (R)2 * (R)c[2] * rho2 + (R)3 * (R)c[3] * rho2 * rho2;
  const R drho2 = (R)2 * r / (rloc * rloc);
  return d_erf + exp((R)-0.5 * rho2) * ((R)-0.5 * poly + dpoly) * drho2;
}

// partials[(k*3 + c) * nblk + block] = sum rho * dV_k/dR_c.
template <typename T>
__global__ void k_local_grad(const T* __restrict__ rho, int N, double L, double h, AtomTable at,
                             double* partials) {
  __shared__ double sh[32];
  const int64_t n3 = (int64_t)N * N * N;
  for (int k = 0; k < at.K; ++k) {
    Acc<T> g[3];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3;
         i += (int64_t)gridDim.x * blockDim.x) {
      const int z = (int)(i % N), y = (int)((i / N) % N), x = (int)(i / ((int64_t)N * N));
      const double dxd = axis_coord(x, L, h) - at.x[k];
      const double dyd = axis_coord(y, L, h) - at.y[k];
      const double dzd = axis_coord(z, L, h) - at.z[k];
      const T dx = (T)dxd, dy = (T)dyd, dz = (T)dzd;
      const T r = sqrt(dx * dx + dy * dy + dz * dz + (T)1e-30);
      const T dv = hgh_dvloc_dr<T>(r, (T)at.Z[k], (T)at.rloc[k], at.c[k]);
      // dV/dR = dV/dr * (-(x - R)/r)
      const T w = -rho[i] * dv / r;
      g[0].add_prod(w, dx);
      g[1].add_prod(w, dy);
      g[2].add_prod(w, dz);
    }
    for (int cc = 0; cc < 3; ++cc) {
      const double v = block_sum(g[cc].value(), sh);
      if (threadIdx.x == 0) partials[(k * 3 + cc) * gridDim.x + blockIdx.x] = v;
    }
  }
}

// d/dR_k of int rho V_soft with V_soft = -Z_k / sqrt(|r - R_k|^2 + eps^2):
// int rho(r) (-Z_k) (r - R_k) / (|r - R_k|^2 + eps^2)^{3/2} dV.
template <typename T>
__global__ void k_softened_grad(const T* __restrict__ rho, int N, double L, double h, AtomTable at,
                                double eps, double* partials) {
  __shared__ double sh[32];
  const int64_t n3 = (int64_t)N * N * N;
  const T e2 = (T)(eps * eps);
  for (int k = 0; k < at.K; ++k) {
    Acc<T> g[3];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3;
         i += (int64_t)gridDim.x * blockDim.x) {
      const int z = (int)(i % N), y = (int)((i / N) % N), x = (int)(i / ((int64_t)N * N));
      const T dx = (T)(axis_coord(x, L, h) - at.x[k]);
      const T dy = (T)(axis_coord(y, L, h) - at.y[k]);
      const T dz = (T)(axis_coord(z, L, h) - at.z[k]);
      const T u = dx * dx + dy * dy + dz * dz + e2;
      const T w = -(T)at.Z[k] * rho[i] / (u * sqrt(u));
      g[0].add_prod(w, dx);
      g[1].add_prod(w, dy);
      g[2].add_prod(w, dz);
    }
    for (int cc = 0; cc < 3; ++cc) {
      const double v = block_sum(g[cc].value(), sh);
      if (threadIdx.x == 0) partials[(k * 3 + cc) * gridDim.x + blockIdx.x] = v;
    }
  }
}

// ---- non-local projectors -------------------------------------------------------

struct ProjParams {
  double ax, ay, az;   // atom position
  int ell, m, power;
  double r, norm;
};

__device__ __forceinline__ double angular(int ell, int m, double hx, double hy, double hz) {
  const double pi = 3.14159265358979323846;
  if (ell == 0) return 1.0 / sqrt(4.0 * pi);
  if (ell == 1) {
    const double c = sqrt(3.0 / (4.0 * pi));
    return c * (m == -1 ? hy : (m == 0 ? hz : hx));
  }
  const double c15 = sqrt(15.0 / (4.0 * pi));
  switch (m) {
    case -2: return c15 * hx * hy;
    case -1: return c15 * hy * hz;
    case 0: return 0.25 * sqrt(5.0 / pi) * (3.0 * hz * hz - 1.0);
    case 1: return c15 * hx * hz;
    default: return 0.25 * sqrt(15.0 / pi) * (hx * hx - hy * hy);
  }
}

// d Y / d hat
__device__ __forceinline__ void angular_grad(int ell, int m, double hx, double hy, double hz,
                                             double* g) {
  const double pi = 3.14159265358979323846;
  g[0] = g[1] = g[2] = 0.0;
  if (ell == 0) return;
  if (ell == 1) {
    const double c = sqrt(3.0 / (4.0 * pi));
    g[m == -1 ? 1 : (m == 0 ? 2 : 0)] = c;
    return;
  }
  const double c15 = sqrt(15.0 / (4.0 * pi));
  switch (m) {
    case -2: g[0] = c15 * hy; g[1] = c15 * hx; break;
    case -1: g[1] = c15 * hz; g[2] = c15 * hy; break;
    case 0: g[2] = 0.25 * sqrt(5.0 / pi) * 6.0 * hz; break;
    case 1: g[0] = c15 * hz; g[2] = c15 * hx; break;
    default: g[0] = 0.25 * sqrt(15.0 / pi) * 2.0 * hx; g[1] = -0.25 * sqrt(15.0 / pi) * 2.0 * hy; break;
  }
}

// p(d) of pseudopotentials.py:265-327, r = sqrt(|d|^2 + 1e-30), hat = d / r.
__device__ __forceinline__ double proj_value(const ProjParams& p, double dx, double dy, double dz) {
  const double r = sqrt(dx * dx + dy * dy + dz * dz + 1e-30);
  const double radial = p.norm * pow(r, (double)p.power) * exp(-(r * r) / (2.0 * p.r * p.r));
  return radial * angular(p.ell, p.m, dx / r, dy / r, dz / r);
}

__device__ __forceinline__ void proj_grad(const ProjParams& p, double dx, double dy, double dz,
                                          double* g) {
  const double r = sqrt(dx * dx + dy * dy + dz * dz + 1e-30);
  const double R = p.norm * pow(r, (double)p.power) * exp(-(r * r) / (2.0 * p.r * p.r));
  const double hx = dx / r, hy = dy / r, hz = dz / r;
  const double Y = angular(p.ell, p.m, hx, hy, hz);
  double gY[3];
  angular_grad(p.ell, p.m, hx, hy, hz, gY);
  const double dRr = (p.power / r - r / (p.r * p.r)) * Y;
  const double d[3] = {dx, dy, dz};
  const double hd = gY[0] * hx + gY[1] * hy + gY[2] * hz;
  for (int c = 0; c < 3; ++c) g[c] = R * (dRr * d[c] / r + (gY[c] - hd * d[c] / r) / r);
}

template <typename T>
__global__ void k_nl_values(T* vals, NlBox b, ProjParams pp, int N, double L, double h) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < b.npts;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int z = b.z0 + (int)(t % b.nz);
    const int y = b.y0 + (int)((t / b.nz) % b.ny);
    const int x = b.x0 + (int)(t / ((int64_t)b.nz * b.ny));
    vals[t] = (T)proj_value(pp, axis_coord(x, L, h) - pp.ax, axis_coord(y, L, h) - pp.ay,
                            axis_coord(z, L, h) - pp.az);
  }
}

__device__ __forceinline__ int64_t box_global(const int* bx, int64_t t, int N) {
  const int nz = bx[5], ny = bx[4];
  const int z = bx[2] + (int)(t % nz);
  const int y = bx[1] + (int)((t / nz) % ny);
  const int x = bx[0] + (int)(t / ((int64_t)nz * ny));
  return ((int64_t)x * N + y) * N + z;
}

// grid (nq, kChunks, nb): partials[(b*nq + q)*kChunks + chunk] = sum p*psi.
// The last block to finish (a ticket counter, the threadfence-reduction
// pattern: no block waits for another) then reduces the partials of every
// (b, q) in the k_finalize_sums order, ov = dV * sum, and forms
// coef[b][q] = sum_j h_ij ov[b][block + j]; it resets the ticket for the next
// launch. One launch instead of overlap + finalize + coefficient launches.
template <typename T>
__global__ void k_nl_overlap(const T* __restrict__ psi, const T* __restrict__ vals, const int* q_atom,
                             const int64_t* q_off, const int* boxes, int N, double* part, double dV,
                             double* ov, double* coef, const int* q_block, const int* q_n, const int* q_i,
                             const double* q_h, unsigned* ticket) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int q = blockIdx.x, chunk = blockIdx.y, b = blockIdx.z, nq = gridDim.x, nb = gridDim.z;
  const int a = q_atom[q];
  const int* bx = boxes + 6 * a;
  const int64_t npts = (int64_t)bx[3] * bx[4] * bx[5];
  const T* pv = vals + q_off[q];
  const T* ps = psi + (int64_t)b * N * N * N;
  Acc<T> acc;
  for (int64_t t = (int64_t)chunk * blockDim.x + threadIdx.x; t < npts;
       t += (int64_t)gridDim.y * blockDim.x)
    acc.add_prod(pv[t], ps[box_global(bx, t, N)]);
  const double v = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) {
    part[((int64_t)b * nq + q) * gridDim.y + chunk] = v;
    __threadfence();   // the partial is visible before the ticket counts this block
    const unsigned total = gridDim.x * gridDim.y * gridDim.z;
    last = atomicAdd(ticket, 1u) == total - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int nqb = nq * nb, nch = gridDim.y;
  for (int j = 0; j < nqb; ++j) {
    double sum = 0.0;
    for (int i = threadIdx.x; i < nch; i += blockDim.x) sum += __ldcg(part + (int64_t)j * nch + i);
    sum = block_sum(sum, sh);
    if (threadIdx.x == 0) ov[j] = sum * dV;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nqb; t += blockDim.x) {
    const int bb = t / nq, qq = t % nq;
    const int blk = q_block[qq], n = q_n[qq], i = q_i[qq];
    double c = 0.0;
    for (int j = 0; j < n; ++j) c += q_h[9 * qq + 3 * i + j] * ov[bb * nq + blk + j];
    coef[t] = c;
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// out[b][box pt] += sum_{q in atom} coef[b][q] * p_q(pt)
// The atom's coefficients (rounded once to the field type) and value offsets
// are staged in shared memory, so no element converts from FP64.
constexpr int kNlAddMaxQ = 64;   // projectors of one atom (HGH: at most 2 (2l+1) per l <= 2)

template <typename T>
__global__ void k_nl_add(T* out, const T* __restrict__ vals, const double* coef, const int64_t* q_off,
                         const int* boxes, int atom, int q0, int nqa, int nq, int N) {
  __shared__ T cf[kNlAddMaxQ];
  __shared__ int64_t off[kNlAddMaxQ];
  const int* bx = boxes + 6 * atom;
  const int64_t npts = (int64_t)bx[3] * bx[4] * bx[5];
  const int b = blockIdx.y;
  for (int k = threadIdx.x; k < nqa; k += blockDim.x) {
    cf[k] = (T)coef[b * nq + q0 + k];
    off[k] = q_off[q0 + k];
  }
  __syncthreads();
  T* o = out + (int64_t)b * N * N * N;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < npts;
       t += (int64_t)gridDim.x * blockDim.x) {
    T s = (T)0;
    for (int k = 0; k < nqa; ++k) s += cf[k] * vals[off[k] + t];
    o[box_global(bx, t, N)] += s;
  }
}

// The whole apply for one vector b in one cluster of kNlCluster CTAs (grid
// (kNlCluster, nb)): each CTA takes every kNlCluster-th stretch of every box,
// reduces its partial overlaps per projector in shared memory, and after a
// cluster barrier every CTA sums the kNlCluster partials of each projector in
// rank order through distributed shared memory (the same sums in every CTA),
// forms coef[q] = sum_j h_ij ov[block + j] and adds sum_q coef[q] p_q to out
// over its share of each atom's box, atom by atom with a cluster barrier in
// between. ov and coef of the vector are also left in global memory.
namespace cg = cooperative_groups;
constexpr int kNlCluster = 8;          // CTAs per vector (the portable cluster size)
constexpr int kNlClThreads = 512;
constexpr int kNlClMaxQ = 64;          // projectors of all atoms
constexpr int kNlQChunk = 8;           // projectors of one atom accumulated per pass over its box
struct NlAtomRange {
  int q0[kMaxAtoms], nq[kMaxAtoms];
};

template <typename T>
__global__ void __cluster_dims__(kNlCluster, 1, 1) __launch_bounds__(kNlClThreads)
    k_nl_apply_cluster(const T* __restrict__ psi, T* out, const T* __restrict__ vals, const int* q_atom,
                       const int64_t* q_off, const int* boxes, const int* q_block, const int* q_n,
                       const int* q_i, const double* q_h, int nq, int K, NlAtomRange ar, int N, double dV,
                       double* ov_out, double* coef_out) {
  cg::cluster_group cl = cg::this_cluster();
  __shared__ double wsum[kNlClMaxQ][kNlClThreads / 32];
  __shared__ double part[kNlClMaxQ];
  __shared__ double ovs[kNlClMaxQ];
  __shared__ T cf[kNlClMaxQ];
  const int rank = (int)cl.block_rank(), b = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int start = rank * blockDim.x + threadIdx.x, stride = kNlCluster * blockDim.x;
  const T* ps = psi + (int64_t)b * N * N * N;
  T* o = out + (int64_t)b * N * N * N;
  // overlaps atom by atom, up to kNlQChunk projectors of one atom per pass over its box: a point's
  // index and psi value serve every projector of the pass (each projector's sum runs over the
  // thread's points in the same order as a pass of its own)
  for (int a = 0; a < K; ++a) {
    const int nqa = ar.nq[a];
    const int* bx = boxes + 6 * a;
    const int nz = bx[5], nyz = bx[4] * bx[5], npts = bx[3] * nyz;
    for (int c0 = 0; c0 < nqa; c0 += kNlQChunk) {
      const int q0 = ar.q0[a] + c0, nc = min(kNlQChunk, nqa - c0);
      const T* pv[kNlQChunk];
      Acc<T> acc[kNlQChunk];
#pragma unroll
      for (int k = 0; k < kNlQChunk; ++k) pv[k] = vals + q_off[q0 + (k < nc ? k : 0)];
      for (int t = start; t < npts; t += stride) {
        const int x = bx[0] + t / nyz, y = bx[1] + (t % nyz) / nz, z = bx[2] + t % nz;
        const T pst = ps[((int64_t)x * N + y) * N + z];
#pragma unroll
        for (int k = 0; k < kNlQChunk; ++k)
          if (k < nc) acc[k].add_prod(pv[k][t], pst);
      }
#pragma unroll
      for (int k = 0; k < kNlQChunk; ++k) {
        if (k >= nc) break;
        double v = acc[k].value();
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) wsum[q0 + k][warp] = v;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    double v = 0.0;
    for (int w = 0; w < nw; ++w) v += wsum[threadIdx.x][w];
    part[threadIdx.x] = v;
  }
  cl.sync();   // every CTA's partial overlaps are in its shared memory
  if (threadIdx.x < nq) {
    double v = 0.0;
    for (int r = 0; r < kNlCluster; ++r) v += cl.map_shared_rank(part, r)[threadIdx.x];
    ovs[threadIdx.x] = v * dV;
  }
  cl.sync();   // the remote reads are done (no CTA leaves while another reads it); ovs is complete
  if (threadIdx.x < nq) {
    const int q = threadIdx.x, blk = q_block[q], n = q_n[q], i = q_i[q];
    double c = 0.0;
    for (int j = 0; j < n; ++j) c += q_h[9 * q + 3 * i + j] * ovs[blk + j];
    cf[q] = (T)c;
    if (rank == 0) {
      ov_out[b * nq + q] = ovs[q];
      coef_out[b * nq + q] = c;
    }
  }
  __syncthreads();
  bool first = true;
  for (int a = 0; a < K; ++a) {
    const int nqa = ar.nq[a];
    if (nqa == 0) continue;
    if (!first) cl.sync();   // the previous atom's adds are done: boxes of two atoms may overlap
    first = false;
    const int q0 = ar.q0[a];
    const int* bx = boxes + 6 * a;
    const int nz = bx[5], nyz = bx[4] * bx[5], npts = bx[3] * nyz;
    for (int t = start; t < npts; t += stride) {
      T v = (T)0;
      for (int k = 0; k < nqa; ++k) v += cf[q0 + k] * vals[q_off[q0 + k] + t];
      const int x = bx[0] + t / nyz, y = bx[1] + (t % nyz) / nz, z = bx[2] + t % nz;
      o[((int64_t)x * N + y) * N + z] += v;
    }
  }
}

// energy = 2 * sum_b sum_q ov[b][q] coef[b][q]
__global__ void k_nl_energy(const double* ov, const double* coef, int n, double* out) {
  __shared__ double sh[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += ov[i] * coef[i];
  v = block_sum(v, sh);
  if (threadIdx.x == 0) out[0] = 2.0 * v;
}

// grid (nq, kChunks, nb): partials of -sum grad_d p * psi  (3 comps)

template <typename T>
__global__ void k_nl_dov(const T* __restrict__ psi, const int* q_atom, const int* boxes, int N,
                         double L, double h, const ProjParams* pps, double* part) {
  __shared__ double sh[32];
  const int q = blockIdx.x, chunk = blockIdx.y, b = blockIdx.z, nq = gridDim.x;
  const ProjParams pp = pps[q];
  const int* bx = boxes + 6 * q_atom[q];
  const int64_t npts = (int64_t)bx[3] * bx[4] * bx[5];
  const T* ps = psi + (int64_t)b * N * N * N;
  double g[3] = {0, 0, 0};
  for (int64_t t = (int64_t)chunk * blockDim.x + threadIdx.x; t < npts;
       t += (int64_t)gridDim.y * blockDim.x) {
    const int z = bx[2] + (int)(t % bx[5]);
    const int y = bx[1] + (int)((t / bx[5]) % bx[4]);
    const int x = bx[0] + (int)(t / ((int64_t)bx[5] * bx[4]));
    double gr[3];
    proj_grad(pp, axis_coord(x, L, h) - pp.ax, axis_coord(y, L, h) - pp.ay,
              axis_coord(z, L, h) - pp.az, gr);
    const double v = (double)ps[((int64_t)x * N + y) * N + z];
    for (int c = 0; c < 3; ++c) g[c] -= gr[c] * v;   // dp/dR = -grad_d p
  }
  for (int c = 0; c < 3; ++c) {
    const double v = block_sum(g[c], sh);
    if (threadIdx.x == 0) part[(((int64_t)b * nq + q) * 3 + c) * gridDim.y + chunk] = v;
  }
}

// grad[atom][c] += 4 * sum_b sum_q coef[b][q] * dov[b][q][c]  (single thread block)
__global__ void k_nl_grad_combine(const double* coef, const double* dov, const int* q_atom, int nq,
                                  int nb, int K, double* grad) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i < 3 * K; ++i) grad[i] = 0.0;
  for (int b = 0; b < nb; ++b)
    for (int q = 0; q < nq; ++q)
      for (int c = 0; c < 3; ++c)
        grad[3 * q_atom[q] + c] += 4.0 * coef[b * nq + q] * dov[((int64_t)b * nq + q) * 3 + c];
}

int make_atoms(AtomTable& at, int K, const double* pos, const double* Z, const double* rloc,
               const double* c) {
  if (K < 0 || K > kMaxAtoms) return fail(GATO_EBADARG, "at most %d atoms (got %d)", kMaxAtoms, K);
  at.K = K;
  for (int k = 0; k < K; ++k) {
    at.x[k] = pos[3 * k];
    at.y[k] = pos[3 * k + 1];
    at.z[k] = pos[3 * k + 2];
    at.Z[k] = Z ? Z[k] : 0.0;
    at.rloc[k] = rloc ? rloc[k] : 1.0;
    for (int i = 0; i < 4; ++i) at.c[k][i] = c ? c[4 * k + i] : 0.0;
  }
  return GATO_OK;
}

ProjParams proj_params(const Nonlocal& nl, const NlProj& p) {
  const NlChannel& ch = nl.ch[p.chan];
  ProjParams pp;
  pp.ax = nl.pos[3 * p.atom];
  pp.ay = nl.pos[3 * p.atom + 1];
  pp.az = nl.pos[3 * p.atom + 2];
  pp.ell = ch.ell;
  pp.m = p.m;
  pp.power = ch.ell + 2 * (p.i - 1);
  pp.r = ch.r;
  const double n = ch.ell + (4.0 * p.i - 1.0) / 2.0;      // pseudopotentials.py:274-276
  pp.norm = sqrt(2.0) / (pow(ch.r, n) * sqrt(tgamma(n)));
  return pp;
}

// <p_q | psi[b]> * dV -> nl.ov
int nl_overlaps(Nonlocal& nl, const void* psi, int nb, cudaStream_t s) {
  dim3 g(nl.nq, Nonlocal::kChunks, nb);
  if (nl.dtype == GATO_F64)
    k_nl_overlap<double><<<g, 256, 0, s>>>((const double*)psi, (const double*)nl.vals, nl.d_q_atom,
                                           nl.d_q_off, nl.d_box, nl.N, nl.part, nl.dV, nl.ov, nl.coef,
                                           nl.d_q_block, nl.d_q_n, nl.d_q_i, nl.d_q_h, nl.ticket);
  else
    k_nl_overlap<float><<<g, 256, 0, s>>>((const float*)psi, (const float*)nl.vals, nl.d_q_atom,
                                          nl.d_q_off, nl.d_box, nl.N, nl.part, nl.dV, nl.ov, nl.coef,
                                          nl.d_q_block, nl.d_q_n, nl.d_q_i, nl.d_q_h, nl.ticket);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

}  // namespace

int nonlocal_apply(Nonlocal& nl, const void* psi, void* out, int nb, cudaStream_t s) {
  if (nl.nq == 0) return GATO_OK;
  if (nb > Nonlocal::kMaxVec) return fail(GATO_EBADARG, "nonlocal: at most %d vectors", Nonlocal::kMaxVec);
  bool small_boxes = true;
  for (int a = 0; a < nl.K; ++a) small_boxes = small_boxes && nl.box[a].npts < (int64_t)1 << 30;
  if (nl.nq <= kNlClMaxQ && nl.K <= kMaxAtoms && small_boxes) {
    // one cluster launch per apply
    NlAtomRange ar{};
    for (int a = 0; a < nl.K; ++a) {
      ar.q0[a] = nl.atom_q0[a];
      ar.nq[a] = nl.atom_nq[a];
    }
    dim3 g(kNlCluster, nb);
    if (nl.dtype == GATO_F64)
      k_nl_apply_cluster<double><<<g, kNlClThreads, 0, s>>>(
          (const double*)psi, (double*)out, (const double*)nl.vals, nl.d_q_atom, nl.d_q_off, nl.d_box,
          nl.d_q_block, nl.d_q_n, nl.d_q_i, nl.d_q_h, nl.nq, nl.K, ar, nl.N, nl.dV, nl.ov, nl.coef);
    else
      k_nl_apply_cluster<float><<<g, kNlClThreads, 0, s>>>(
          (const float*)psi, (float*)out, (const float*)nl.vals, nl.d_q_atom, nl.d_q_off, nl.d_box,
          nl.d_q_block, nl.d_q_n, nl.d_q_i, nl.d_q_h, nl.nq, nl.K, ar, nl.N, nl.dV, nl.ov, nl.coef);
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }
  GATO_TRY(nl_overlaps(nl, psi, nb, s));
  for (int a = 0; a < nl.K; ++a) {
    if (nl.atom_nq[a] == 0) continue;
    if (nl.atom_nq[a] > kNlAddMaxQ) return fail(GATO_EUNSUPPORTED, "nonlocal: more than %d projectors on one atom", kNlAddMaxQ);
    const int64_t npts = nl.box[a].npts;
    dim3 g(grid_for(npts, 256, 152 * 4), nb);
    if (nl.dtype == GATO_F64)
      k_nl_add<double><<<g, 256, 0, s>>>((double*)out, (const double*)nl.vals, nl.coef, nl.d_q_off,
                                         nl.d_box, a, nl.atom_q0[a], nl.atom_nq[a], nl.nq, nl.N);
    else
      k_nl_add<float><<<g, 256, 0, s>>>((float*)out, (const float*)nl.vals, nl.coef, nl.d_q_off,
                                        nl.d_box, a, nl.atom_q0[a], nl.atom_nq[a], nl.nq, nl.N);
    GATO_LAUNCH_TRY();
  }
  return GATO_OK;
}

int nonlocal_energy(Nonlocal& nl, const void* psi, int nb, double* energy_dev, cudaStream_t s) {
  if (nl.nq == 0) {
    GATO_CUDA_TRY(cudaMemsetAsync(energy_dev, 0, sizeof(double), s));
    return GATO_OK;
  }
  if (nb > Nonlocal::kMaxVec) return fail(GATO_EBADARG, "nonlocal: at most %d vectors", Nonlocal::kMaxVec);
  GATO_TRY(nl_overlaps(nl, psi, nb, s));
  k_nl_energy<<<1, 256, 0, s>>>(nl.ov, nl.coef, nl.nq * nb, energy_dev);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

}  // namespace gato

using namespace gato;

extern "C" int gato_softened_coulomb(int dtype, void* V, int N, double L, int K,
                                     const double* pos_host, const double* Z_host, double eps,
                                     void* stream) {
  if (!V || N < 1 || L <= 0 || (K > 0 && (!pos_host || !Z_host)))
    return fail(GATO_EBADARG, "gato_softened_coulomb: bad arguments");
  AtomTable at;
  GATO_TRY(make_atoms(at, K, pos_host, Z_host, nullptr, nullptr));
  cudaStream_t s = as_stream(stream);
  const double h = L / N;
  const int64_t n3 = (int64_t)N * N * N;
  if (dtype == GATO_F64) k_softened<double><<<grid_for(n3, 256), 256, 0, s>>>((double*)V, N, L, h, at, eps);
  else k_softened<float><<<grid_for(n3, 256), 256, 0, s>>>((float*)V, N, L, h, at, eps);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

extern "C" int gato_hgh_local(int dtype, void* V, int N, double L, int K, const double* pos_host,
                              const double* Zion_host, const double* rloc_host,
                              const double* c_host, void* stream) {
  if (!V || N < 1 || L <= 0 || (K > 0 && (!pos_host || !Zion_host || !rloc_host || !c_host)))
    return fail(GATO_EBADARG, "gato_hgh_local: bad arguments");
  AtomTable at;
  GATO_TRY(make_atoms(at, K, pos_host, Zion_host, rloc_host, c_host));
  cudaStream_t s = as_stream(stream);
  const double h = L / N;
  const int64_t n3 = (int64_t)N * N * N;
  if (dtype == GATO_F64) k_hgh_local<double><<<grid_for(n3, 256), 256, 0, s>>>((double*)V, N, L, h, at);
  else k_hgh_local<float><<<grid_for(n3, 256), 256, 0, s>>>((float*)V, N, L, h, at);
  GATO_LAUNCH_TRY();
  return GATO_OK;
}

extern "C" int gato_hgh_local_grad(int dtype, const void* rho, int N, double L, int K,
                                   const double* pos_host, const double* Zion_host,
                                   const double* rloc_host, const double* c_host,
                                   double* grad_host, void* stream) {
  if (!rho || N < 1 || L <= 0 || K < 1 || !pos_host || !Zion_host || !rloc_host || !c_host ||
      !grad_host)
    return fail(GATO_EBADARG, "gato_hgh_local_grad: bad arguments");
  AtomTable at;
  GATO_TRY(make_atoms(at, K, pos_host, Zion_host, rloc_host, c_host));
  cudaStream_t s = as_stream(stream);
  const double h = L / N;
  const int nblk = kRedBlocks;
  double* part = (double*)stream_scratch(s, (size_t)(3 * K * nblk + 3 * K) * sizeof(double));
  if (!part) return fail(GATO_ENOMEM, "scratch");
  double* res = part + 3 * K * nblk;
  if (dtype == GATO_F64) k_local_grad<double><<<nblk, 256, 0, s>>>((const double*)rho, N, L, h, at, part);
  else k_local_grad<float><<<nblk, 256, 0, s>>>((const float*)rho, N, L, h, at, part);
  GATO_LAUNCH_TRY();
  GATO_TRY(finalize_sums(part, 3 * K, nblk, h * h * h, res, s));
  std::vector<double> g(3 * K);
  GATO_CUDA_TRY(cudaMemcpyAsync(g.data(), res, 3 * K * sizeof(double), cudaMemcpyDeviceToHost, s));
  GATO_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < 3 * K; ++i) grad_host[i] += g[i];
  return GATO_OK;
}

extern "C" int gato_softened_coulomb_grad(int dtype, const void* rho, int N, double L, int K,
                                          const double* pos_host, const double* Z_host, double eps,
                                          double* grad_host, void* stream) {
  if (!rho || N < 1 || L <= 0 || K < 1 || !pos_host || !Z_host || !grad_host)
    return fail(GATO_EBADARG, "gato_softened_coulomb_grad: bad arguments");
  AtomTable at;
  GATO_TRY(make_atoms(at, K, pos_host, Z_host, nullptr, nullptr));
  cudaStream_t s = as_stream(stream);
  const double h = L / N;
  const int nblk = kRedBlocks;
  double* part = (double*)stream_scratch(s, (size_t)(3 * K * nblk + 3 * K) * sizeof(double));
  if (!part) return fail(GATO_ENOMEM, "scratch");
  double* res = part + 3 * K * nblk;
  if (dtype == GATO_F64)
    k_softened_grad<double><<<nblk, 256, 0, s>>>((const double*)rho, N, L, h, at, eps, part);
  else
    k_softened_grad<float><<<nblk, 256, 0, s>>>((const float*)rho, N, L, h, at, eps, part);
  GATO_LAUNCH_TRY();
  GATO_TRY(finalize_sums(part, 3 * K, nblk, h * h * h, res, s));
  std::vector<double> g(3 * K);
  GATO_CUDA_TRY(cudaMemcpyAsync(g.data(), res, 3 * K * sizeof(double), cudaMemcpyDeviceToHost, s));
  GATO_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < 3 * K; ++i) grad_host[i] += g[i];
  return GATO_OK;
}

extern "C" int gato_nonlocal_create(int dtype, int N, double L, int K, const double* pos_host,
                                    const int* nch_host, const int* ell_host, const double* r_host,
                                    const int* n_host, const double* h_host, double cut_sigmas,
                                    gato_nonlocal_t* out) {
  if (!out || N < 1 || L <= 0 || K < 0 || (K > 0 && (!pos_host || !nch_host)) || cut_sigmas <= 0)
    return fail(GATO_EBADARG, "gato_nonlocal_create: bad arguments");
  if (dtype != GATO_F64 && dtype != GATO_F32) return fail(GATO_EBADARG, "bad dtype %d", dtype);
  auto* w = new gato_nonlocal();
  Nonlocal& nl = w->n;
  nl.dtype = dtype;
  nl.N = N;
  nl.L = L;
  nl.h = L / N;
  nl.dV = nl.h * nl.h * nl.h;
  nl.K = K;
  nl.pos.assign(pos_host, pos_host + 3 * K);
  int c = 0;
  for (int a = 0; a < K; ++a) {
    nl.atom_q0.push_back((int)nl.proj.size());
    double rmax = 0;
    for (int k = 0; k < nch_host[a]; ++k, ++c) {
      NlChannel ch;
      ch.atom = a;
      ch.ell = ell_host[c];
      ch.n = n_host[c];
      ch.r = r_host[c];
      for (int i = 0; i < 9; ++i) ch.h[i] = h_host[9 * c + i];
      if (ch.ell < 0 || ch.ell > 2) {
        delete w;
        return fail(GATO_EUNSUPPORTED, "Real Y_{%d,m} not implemented (need l <= 2).", ch.ell);
      }
      if (ch.n < 1 || ch.n > 3 || ch.r <= 0) {
        delete w;
        return fail(GATO_EBADARG, "nonlocal: bad channel (n=%d r=%g)", ch.n, ch.r);
      }
      rmax = std::max(rmax, ch.r);
      const int chan = (int)nl.ch.size();
      nl.ch.push_back(ch);
      for (int m = -ch.ell; m <= ch.ell; ++m)
        for (int i = 1; i <= ch.n; ++i) nl.proj.push_back({a, chan, m, i, 0});
    }
    nl.atom_nq.push_back((int)nl.proj.size() - nl.atom_q0.back());
    NlBox b{0, 0, 0, 0, 0, 0, 0};
    if (nl.atom_nq.back() > 0) {
      const double rc = cut_sigmas * rmax;
      int lo[3], hi[3];
      for (int d = 0; d < 3; ++d) {
        const double p = nl.pos[3 * a + d];
        // grid points x_i = -L/2 + (i + 1/2) h within [p - rc, p + rc]
        lo[d] = std::max(0, (int)std::ceil((p - rc + L / 2) / nl.h - 0.5));
        hi[d] = std::min(N - 1, (int)std::floor((p + rc + L / 2) / nl.h - 0.5));
        if (hi[d] < lo[d]) hi[d] = lo[d] - 1;
      }
      b = {lo[0], lo[1], lo[2], hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1, 0};
      if (b.nx <= 0 || b.ny <= 0 || b.nz <= 0) b = {0, 0, 0, 0, 0, 0, 0};
      b.npts = (int64_t)b.nx * b.ny * b.nz;
    }
    nl.box.push_back(b);
  }
  nl.nq = (int)nl.proj.size();
  if (nl.nq > 64) {
    delete w;
    return fail(GATO_EUNSUPPORTED, "nonlocal: at most 64 projectors (got %d)", nl.nq);
  }
  // empty boxes (atom outside the grid) contribute nothing: drop their projectors' points
  std::vector<int> q_atom, q_block, q_n, q_i;
  std::vector<int64_t> q_off;
  std::vector<double> q_h;
  std::vector<int> boxes;
  int64_t off = 0;
  for (int q = 0; q < nl.nq; ++q) {
    NlProj& p = nl.proj[q];
    p.off = off;
    off += nl.box[p.atom].npts;
    const NlChannel& ch = nl.ch[p.chan];
    q_atom.push_back(p.atom);
    q_off.push_back(p.off);
    q_block.push_back(q - (p.i - 1));
    q_n.push_back(ch.n);
    q_i.push_back(p.i - 1);
    for (int i = 0; i < 9; ++i) q_h.push_back(ch.h[i]);
  }
  for (int a = 0; a < K; ++a) {
    const NlBox& b = nl.box[a];
    int v[6] = {b.x0, b.y0, b.z0, b.nx, b.ny, b.nz};
    boxes.insert(boxes.end(), v, v + 6);
  }
  nl.nvals = off;
  const size_t es = dtype == GATO_F64 ? 8 : 4;
  int st = GATO_OK;
  auto alloc = [&](void** p, size_t bytes) {
    if (st != GATO_OK) return;
    if (cudaMalloc(p, bytes < 8 ? 8 : bytes) != cudaSuccess)
      st = fail(GATO_ENOMEM, "nonlocal: allocation of %zu bytes failed", bytes);
  };
  auto up = [&](void* d, const void* h, size_t bytes) {
    if (st != GATO_OK || bytes == 0) return;
    if (cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
      st = fail(GATO_ECUDA, "nonlocal: upload failed");
  };
  const int nq = nl.nq;
  alloc(&nl.vals, (size_t)std::max<int64_t>(off, 1) * es);
  alloc((void**)&nl.d_q_atom, nq * sizeof(int));
  alloc((void**)&nl.d_q_off, nq * sizeof(int64_t));
  alloc((void**)&nl.d_q_block, nq * sizeof(int));
  alloc((void**)&nl.d_q_n, nq * sizeof(int));
  alloc((void**)&nl.d_q_i, nq * sizeof(int));
  alloc((void**)&nl.d_q_h, nq * 9 * sizeof(double));
  alloc((void**)&nl.d_box, std::max(K, 1) * 6 * sizeof(int));
  const size_t nvq = (size_t)Nonlocal::kMaxVec * std::max(nq, 1);
  alloc((void**)&nl.ov, nvq * sizeof(double));
  alloc((void**)&nl.coef, nvq * sizeof(double));
  alloc((void**)&nl.dov, nvq * 3 * sizeof(double));
  alloc((void**)&nl.part, nvq * 3 * Nonlocal::kChunks * sizeof(double));
  alloc((void**)&nl.ticket, sizeof(unsigned));
  if (nl.ticket && cudaMemset(nl.ticket, 0, sizeof(unsigned)) != cudaSuccess)
    st = fail(GATO_ECUDA, "nonlocal: ticket reset failed");
  up(nl.d_q_atom, q_atom.data(), nq * sizeof(int));
  up(nl.d_q_off, q_off.data(), nq * sizeof(int64_t));
  up(nl.d_q_block, q_block.data(), nq * sizeof(int));
  up(nl.d_q_n, q_n.data(), nq * sizeof(int));
  up(nl.d_q_i, q_i.data(), nq * sizeof(int));
  up(nl.d_q_h, q_h.data(), nq * 9 * sizeof(double));
  up(nl.d_box, boxes.data(), boxes.size() * sizeof(int));
  for (int q = 0; q < nq && st == GATO_OK; ++q) {
    const NlProj& p = nl.proj[q];
    const NlBox& b = nl.box[p.atom];
    if (b.npts == 0) continue;
    ProjParams pp = proj_params(nl, p);
    if (dtype == GATO_F64)
      k_nl_values<double><<<grid_for(b.npts, 256), 256>>>((double*)nl.vals + p.off, b, pp, N, L, nl.h);
    else
      k_nl_values<float><<<grid_for(b.npts, 256), 256>>>((float*)nl.vals + p.off, b, pp, N, L, nl.h);
    if (cudaGetLastError() != cudaSuccess) st = fail(GATO_ECUDA, "nonlocal: value kernel failed");
  }
  if (st == GATO_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(GATO_ECUDA, "nonlocal: sync failed");
  if (st != GATO_OK) {
    gato_nonlocal_destroy(w);
    return st;
  }
  *out = w;
  return GATO_OK;
}

extern "C" int gato_nonlocal_destroy(gato_nonlocal_t w) {
  if (!w) return GATO_OK;
  Nonlocal& nl = w->n;
  free_after_pending({nl.vals, nl.d_q_atom, nl.d_q_off, nl.d_q_block, nl.d_q_n, nl.d_q_i, nl.d_q_h, nl.d_box,
                      nl.ov, nl.coef, nl.dov, nl.part, nl.ticket});
  delete w;
  return GATO_OK;
}

extern "C" int gato_nonlocal_apply(gato_nonlocal_t w, const void* psi, void* out, int nb,
                                   void* stream) {
  if (!w || !psi || !out || nb < 1) return fail(GATO_EBADARG, "gato_nonlocal_apply: bad arguments");
  return nonlocal_apply(w->n, psi, out, nb, as_stream(stream));
}

extern "C" int gato_nonlocal_energy(gato_nonlocal_t w, const void* psi, int nb, double* e_dev,
                                    void* stream) {
  if (!w || !psi || !e_dev || nb < 1) return fail(GATO_EBADARG, "gato_nonlocal_energy: bad arguments");
  return nonlocal_energy(w->n, psi, nb, e_dev, as_stream(stream));
}

extern "C" int gato_nonlocal_grad(gato_nonlocal_t w, const void* orbitals, int n, double* grad_host,
                                  void* stream) {
  if (!w || !orbitals || n < 1 || !grad_host) return fail(GATO_EBADARG, "gato_nonlocal_grad: bad arguments");
  Nonlocal& nl = w->n;
  if (nl.nq == 0) return GATO_OK;
  if (n > Nonlocal::kMaxVec) return fail(GATO_EBADARG, "nonlocal: at most %d vectors", Nonlocal::kMaxVec);
  cudaStream_t s = as_stream(stream);
  GATO_TRY(nl_overlaps(nl, orbitals, n, s));
  std::vector<ProjParams> pps(nl.nq);
  for (int q = 0; q < nl.nq; ++q) pps[q] = proj_params(nl, nl.proj[q]);
  ProjParams* d_pp = (ProjParams*)stream_scratch(s, nl.nq * sizeof(ProjParams) + 3 * nl.K * sizeof(double) + 64);
  if (!d_pp) return fail(GATO_ENOMEM, "scratch");
  double* d_grad = (double*)((char*)d_pp + ((nl.nq * sizeof(ProjParams) + 15) / 16) * 16);
  GATO_CUDA_TRY(cudaMemcpyAsync(d_pp, pps.data(), nl.nq * sizeof(ProjParams), cudaMemcpyHostToDevice, s));
  dim3 g(nl.nq, Nonlocal::kChunks, n);
  if (nl.dtype == GATO_F64)
    k_nl_dov<double><<<g, 256, 0, s>>>((const double*)orbitals, nl.d_q_atom, nl.d_box, nl.N, nl.L, nl.h, d_pp, nl.part);
  else
    k_nl_dov<float><<<g, 256, 0, s>>>((const float*)orbitals, nl.d_q_atom, nl.d_box, nl.N, nl.L, nl.h, d_pp, nl.part);
  GATO_LAUNCH_TRY();
  GATO_TRY(finalize_sums(nl.part, nl.nq * n * 3, Nonlocal::kChunks, nl.dV, nl.dov, s));
  k_nl_grad_combine<<<1, 32, 0, s>>>(nl.coef, nl.dov, nl.d_q_atom, nl.nq, n, nl.K, d_grad);
  GATO_LAUNCH_TRY();
  std::vector<double> g3(3 * nl.K);
  GATO_CUDA_TRY(cudaMemcpyAsync(g3.data(), d_grad, 3 * nl.K * sizeof(double), cudaMemcpyDeviceToHost, s));
  GATO_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < 3 * nl.K; ++i) grad_host[i] += g3[i];
  return GATO_OK;
}
