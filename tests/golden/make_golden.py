"""Generate tests/golden/golden.npz from the CPU oracle.

The reference (JAX) cannot run here, so the committed vectors are the FP64
NumPy restatement's outputs on small seeded inputs; the restatement itself is
pinned to the reference's known-answer tests (tests/test_oracle_kats.py).
Run: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import gato_np as o  # noqa: E402


def water_case(N=16, L=10.0, seed=7):
    """Water at a jittered geometry with 4 seeded smooth orbitals."""
    g = o.Grid3D(N, L)
    rng = np.random.default_rng(seed)
    nuc = o.water_initial_geometry(1.81, 104.5)
    nuc = o.Nuclei(nuc.positions + rng.uniform(-0.05, 0.05, (3, 3)), nuc.charges)
    X, Y, Z = g.coords()
    orbs = []
    for k in range(4):
        c = rng.uniform(-0.6, 0.6, 3)
        a = rng.uniform(0.4, 0.9)
        w = rng.uniform(-0.3, 0.3, 3)
        poly = 1.0 + w[0] * X + w[1] * Y + w[2] * Z
        orbs.append(np.exp(-a * ((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2)) * poly)
    orbs = np.stack(orbs)
    # Gram-Schmidt with the grid metric, so the block is orthonormal
    for i in range(4):
        for j in range(i):
            orbs[i] -= np.sum(orbs[i] * orbs[j]) * g.dV * orbs[j]
        orbs[i] /= np.sqrt(np.sum(orbs[i] ** 2) * g.dV)
    return g, nuc, orbs


def main():
    out = {}
    rng = np.random.default_rng(0)
    g = o.Grid3D(16, 5.0)
    psi = rng.standard_normal(g.shape)
    out["stencil_psi"] = psi
    for order in (2, 4):
        for b in ("dirichlet", "periodic"):
            out[f"stencil_lap_{order}_{b}"] = o.laplacian(psi, g.h, b, order)

    g = o.Grid3D(16, 8.0)
    X, Y, Z = g.coords()
    rho = (0.8 / np.pi) ** 1.5 * np.exp(-0.8 * ((X - 0.5) ** 2 + Y ** 2 + Z ** 2))
    out["hartree_rho"] = rho
    out["hartree_J"] = o.hartree_potential(rho, g)
    out["hartree_E"] = np.array(o.hartree_energy(rho, g))

    g, nuc, orbs = water_case()
    elements = o.water_hgh_elements()
    V_loc = o.hgh_local_potential(nuc, elements, g)
    nl = lambda p: o.hgh_nonlocal_apply(p, nuc, elements, g)  # noqa: E731
    V_H = o.hartree_potential(o._density(np.moveaxis(orbs, 0, -1)), g)
    out["water_positions"] = nuc.positions
    out["water_orbitals"] = orbs
    out["water_V_loc"] = V_loc
    out["water_block_fock"] = o.fock_apply_block(orbs, V_loc + V_H, g, order=4, nl=nl)
    t = o.decompose_rhf_energy(np.moveaxis(orbs, 0, -1), V_loc, g, V_nl_apply=nl)
    out["water_terms"] = np.array([t.kinetic, t.v_ext, t.v_nl, t.hartree, t.exchange])
    out["water_grad"] = o.bo_grad_positions(nuc.positions, nuc.charges, np.moveaxis(orbs, 0, -1), elements, g)

    g = o.Grid3D(16, 10.0)
    H = o.Hamiltonian(g, o.harmonic_oscillator(g), order=4)
    X, Y, Z = g.coords()
    res = o.lanczos(H, np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * (1 + 0.1 * (X + Y + Z)), 30, 3)
    out["lanczos_ho_evals"] = res.eigenvalues
    out["lanczos_ho_alphas"] = res.alphas
    out["lanczos_ho_betas"] = res.betas

    g = o.Grid3D(24, 8.0)
    res = o.scf_rhf(o.softened_coulomb(g, Z=2.0), g, 1, max_iters=6, tol=1e-12, mixing=0.7, order=4,
                    lanczos_iters=30)
    out["he24_history"] = np.array(res.energy_history)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
