"""End-to-end checks of the benchmark workloads on the GPU.

hydrogen: 64^3, L = 20, 7-point Laplacian, softened Coulomb (a = 0.1), Lanczos m = 80 from a seeded
          uniform start -> E0 and psi0 against the FP64 oracle.
helium:   RHF SCF, 96^3, L = 16, 13-point Laplacian, Z = 2, softening 0.1 for V_ext and the
          Hartree/exchange kernel, Gaussian + 1e-3 noise start, mixing 0.5, tol 1e-8, <= 30 iterations:
          FP64 path against the oracle iteration by iteration, mixed against FP64 at convergence.
water:    H2O RHF with HGH at h = 0.25 (64^3 here; the 128^3 case is the benchmark) -> mixed against
          FP64 at convergence, FP64 against the oracle on the first iteration.
forces:   Hellmann-Feynman forces of the mixed path against FP64 central differences (1e-3 bohr) and
          a few Adam steps that lower the energy.
"""
import math

import numpy as np
import pytest
import torch

from oracle import gato_np as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


def dev(x, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x)).to("cuda", dtype)


def test_hydrogen64_lanczos():
    from gato_gb300.grid import Grid3D
    from gato_gb300.hamiltonian import Hamiltonian
    from gato_gb300.potentials import softened_coulomb
    from gato_gb300.solvers.lanczos import lanczos
    og, g = o.Grid3D(64, 20.0), Grid3D(64, 20.0)
    psi0 = np.random.default_rng(0).uniform(0.0, 1.0, og.shape)
    ref = o.lanczos(o.Hamiltonian(og, o.softened_coulomb(og, 1.0, 0.1), order=2), psi0, 80, 1)
    res = {}
    for prec, dt in (("fp64", torch.float64), ("mixed", torch.float32)):
        H = Hamiltonian(g, softened_coulomb(g, 1.0, 0.1, dtype=dt), order=2)
        res[prec] = lanczos(H, dev(psi0, dt), 80, 1)
    e64 = float(res["fp64"].eigenvalues[0])
    assert abs(e64 - ref.eigenvalues[0]) < 1e-10
    ov = abs(float(np.sum(res["fp64"].eigenstates[..., 0].cpu().numpy() * ref.eigenstates[..., 0]) * og.dV))
    assert abs(ov - 1.0) < 1e-8
    assert abs(float(res["mixed"].eigenvalues[0]) - e64) < 1e-6


def _helium_inputs(N=96, L=16.0, seed=3):
    og = o.Grid3D(N, L)
    X, Y, Z = og.coords()
    phi0 = np.exp(-(X * X + Y * Y + Z * Z)) + 1e-3 * np.random.default_rng(seed).standard_normal(og.shape)
    return og, phi0


HE_KW = dict(mixing=0.5, order=4, epsilon=0.1)


def test_helium_first_iteration_vs_oracle():
    from gato_gb300.grid import Grid3D
    from gato_gb300.potentials import softened_coulomb
    from gato_gb300.scf import scf_rhf
    og, phi0 = _helium_inputs()
    g = Grid3D(og.N, og.L)
    ref = o.scf_rhf(o.softened_coulomb(og, 2.0, 0.1), og, 1, initial_orbitals=phi0[..., None], max_iters=1,
                    tol=1e-8, **HE_KW)
    r1 = scf_rhf(softened_coulomb(g, 2.0, 0.1), g, 1, initial_orbitals=dev(phi0)[..., None], max_iters=1,
                 tol=1e-8, **HE_KW)
    assert abs(r1.energy_history[0] - ref.energy_history[0]) < 1e-10


def _helium_mixed_vs_fp64(N, L):
    from gato_gb300.grid import Grid3D
    from gato_gb300.potentials import softened_coulomb
    from gato_gb300.scf import scf_rhf
    og, phi0 = _helium_inputs(N, L)
    g = Grid3D(N, L)
    full = {}
    for prec in ("fp64", "mixed"):
        dt = torch.float64 if prec == "fp64" else torch.float32
        full[prec] = scf_rhf(softened_coulomb(g, 2.0, 0.1), g, 1,
                             initial_orbitals=dev(phi0, dt)[..., None], max_iters=30, tol=1e-8,
                             precision=prec, **HE_KW)
    assert full["fp64"].converged and full["mixed"].n_iters <= 30
    assert abs(full["mixed"].energy - full["fp64"].energy) < 1e-6, (full["mixed"].energy, full["fp64"].energy)
    return full


def test_helium64_mixed_vs_fp64():
    _helium_mixed_vs_fp64(64, 16.0)


def test_helium96_mixed_vs_fp64():
    """The helium workload at its own size (96^3, ~4 s of GPU time for both precisions)."""
    _helium_mixed_vs_fp64(96, 16.0)


def _water(N, h, seed=11):
    from gato_gb300.geometry import Nuclei
    from gato_gb300.physics.water import water_initial_geometry
    nuc = water_initial_geometry(1.81, 104.5)
    jit = torch.tensor(np.random.default_rng(seed).uniform(-0.05, 0.05, (3, 3)))
    return Nuclei(nuc.positions + jit, nuc.charges)


def test_water_scf_mixed_vs_fp64():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import solve_rhf_at_geometry, water_hgh_elements
    N, h = 64, 0.25
    g = Grid3D(N, N * h)
    nuc = _water(N, h)
    el = water_hgh_elements()
    # converge both paths well below the 1e-6 Ha comparison so the difference is precision, not SCF stopping
    p64 = solve_rhf_at_geometry(nuc, el, g, precision="fp64", tol=1e-9, max_iters=80)
    p32 = solve_rhf_at_geometry(nuc, el, g, precision="mixed", tol=1e-9, max_iters=80)
    assert p64.converged
    assert abs(p32.energy - p64.energy) < 1e-6, (p32.energy, p64.energy)
    # Ritz values move at first order with the density (the energy at second order), so an SCF
    # stopped at |dE| < 1e-9 leaves them ~2e-5 Ha from self-consistency on either path
    assert np.max(np.abs(p32.orbital_energies.cpu().numpy() - p64.orbital_energies.cpu().numpy())) < 1e-4
    assert -25.0 < p64.energy < -12.0
    # precision proper: the FP32 and FP64 Fock operators on the same orbitals
    rq = {dt: _fock_rayleigh(p32.orbitals, nuc, el, g, dt) for dt in (torch.float32, torch.float64)}
    assert np.max(np.abs(rq[torch.float32] - rq[torch.float64])) < 1e-6, rq


def _fock_rayleigh(orbitals, nuc, el, g, dtype):
    """<phi_i|F|phi_i> / <phi_i|phi_i> with F built in ``dtype`` from these orbitals."""
    from gato_gb300.pseudopotentials import hgh_local_potential, nonlocal_for
    from gato_gb300.scf import Operator, _density_fields, pair_fields, to_fields
    from gato_gb300.solvers.poisson import get_plan
    n = orbitals.shape[-1]
    f = to_fields(orbitals).to(dtype).contiguous()
    f64 = f.to(torch.float64)
    V = hgh_local_potential(nuc, el, g, torch.float64) + get_plan(g.N, g.h, g.h / 2, torch.float64).potential(
        _density_fields(f64))
    op = Operator(g, dtype, 4, "dirichlet")
    op.set_potential(V.to(dtype).contiguous())
    op.set_nonlocal(nonlocal_for(nuc, el, g, dtype))
    op.set_exchange(get_plan(g.N, g.h, g.h / 2, dtype, pair_fields(n)), f)
    Ff = op.apply_block().to(torch.float64)
    return ((f64 * Ff).flatten(1).sum(1) / (f64 * f64).flatten(1).sum(1)).cpu().numpy()


def test_water_first_iteration_vs_oracle():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import solve_rhf_at_geometry, water_hgh_elements
    N, h = 48, 0.3
    g, og = Grid3D(N, N * h), o.Grid3D(N, N * h)
    nuc = _water(N, h)
    onuc = o.Nuclei(nuc.positions.numpy(), nuc.charges.numpy())
    ref = o.solve_rhf_at_geometry(onuc, o.water_hgh_elements(), og, max_iters=1, lanczos_iters=60)
    got = solve_rhf_at_geometry(nuc, water_hgh_elements(), g, max_iters=1, lanczos_iters=60)
    assert abs(got.energy - ref.energy) < 1e-10, (got.energy, ref.energy)
    assert np.max(np.abs(got.orbital_energies.cpu().numpy() - ref.orbital_energies)) < 1e-10


def test_water_forces_against_fd_and_adam():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import (bo_energy, hellmann_feynman_force, optimize_water_geometry,
                                          solve_rhf_at_geometry, water_hgh_elements)
    from gato_gb300.scf import to_fields
    N, h = 48, 0.3
    g = Grid3D(N, N * h)
    el = water_hgh_elements()
    rng = np.random.default_rng(4)
    R, ang = rng.uniform(1.5, 2.3), rng.uniform(90.0, 130.0)
    from gato_gb300.physics.water import water_initial_geometry
    nuc = water_initial_geometry(R, ang)
    p = solve_rhf_at_geometry(nuc, el, g, precision="mixed")
    F = hellmann_feynman_force(p, el, g).numpy()
    orb64 = to_fields(p.orbitals).to(torch.float64)
    d = 1e-3
    worst = 0.0
    for atom in range(3):
        for ax in range(3):
            pp, pm = p.nuclei.positions.clone(), p.nuclei.positions.clone()
            pp[atom, ax] += d
            pm[atom, ax] -= d
            fd = -(float(bo_energy(pp, p.nuclei.charges, orb64.permute(1, 2, 3, 0), el, g))
                   - float(bo_energy(pm, p.nuclei.charges, orb64.permute(1, 2, 3, 0), el, g))) / (2 * d)
            worst = max(worst, abs(F[atom, ax] - fd))
            assert F[atom, ax] == pytest.approx(fd, rel=1e-3, abs=1e-4)
    # mixed-path analytic forces against FP64 central differences (the 1e-5 Ha/bohr target)
    assert worst < 1e-5, worst
    res = optimize_water_geometry(nuc, el, g, geom_steps=3, learning_rate=0.02, verbose=False, precision="mixed")
    assert res.final.energy <= p.energy + 1e-4
