// HGH non-local projector set (internal API).
#pragma once
#include <vector>

#include "common.cuh"

namespace gato {

struct NlChannel {
  int atom, ell, n;     // n radial projectors
  double r;             // r_l
  double h[9];          // symmetric n x n (row-major 3x3 storage)
};

// One (atom, channel, m, i) projector.
struct NlProj {
  int atom, chan, m, i;     // i is 1-based as in the HGH paper
  int64_t off;              // offset of its values in the value arrays
};

struct NlBox {
  int x0, y0, z0, nx, ny, nz;
  int64_t npts;
};

struct Nonlocal {
  int dtype = GATO_F64;
  int N = 0;
  double L = 0, h = 0, dV = 0;
  int K = 0;
  std::vector<double> pos;          // K x 3
  std::vector<NlChannel> ch;
  std::vector<NlProj> proj;
  std::vector<NlBox> box;           // per atom (npts = 0: no projectors)
  std::vector<int> atom_q0, atom_nq;  // projector range of each atom
  int nq = 0;
  int64_t nvals = 0;
  void* vals = nullptr;             // projector values (dtype), concatenated
  // device copies of the projector metadata
  int* d_q_atom = nullptr;          // per q: atom
  int64_t* d_q_off = nullptr;       // per q: value offset
  int* d_q_block = nullptr;         // per q: first projector of its (atom, chan, m) block
  int* d_q_n = nullptr;             // per q: block size n
  int* d_q_i = nullptr;             // per q: index within block (0-based)
  double* d_q_h = nullptr;          // per q: the 9 h entries of its channel
  int* d_box = nullptr;             // per atom: x0 y0 z0 nx ny nz
  // workspace (sized for kMaxVec vectors)
  double* ov = nullptr;             // [vec][q]
  double* coef = nullptr;           // [vec][q]
  double* part = nullptr;           // partials
  double* dov = nullptr;            // [vec][q][3]
  unsigned* ticket = nullptr;       // blocks done in the running overlap launch (0 between launches)
  static constexpr int kMaxVec = 16;
  static constexpr int kChunks = 32;  // partial sums per projector box
};

int nonlocal_apply(Nonlocal& nl, const void* psi, void* out, int nb, cudaStream_t s);
int nonlocal_energy(Nonlocal& nl, const void* psi, int nb, double* energy_dev, cudaStream_t s);

}  // namespace gato

struct gato_nonlocal {
  gato::Nonlocal n;
};
