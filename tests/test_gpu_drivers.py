"""The molecule drivers beside water (physics/lih.py, hcl.py, h2.py, helium.py of the reference).

Each mirrors the reference's own test (tests/test_lih.py, test_hcl.py, test_h2.py): a bound single
point, the hand-written adjoint force against a central difference of the BO energy at fixed
orbitals, and a geometry optimisation that moves toward equilibrium; plus parity with the FP64
oracle on the first SCF iteration and on the softened-Coulomb force reduction.
"""
import numpy as np
import pytest
import torch

from oracle import gato_np as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


def _fd_z(bo, point, *args):
    """Central difference of the BO energy in z of atom 1 at fixed orbitals, evaluated in FP64."""
    d = 1e-3
    orb = point.orbitals.to(torch.float64)
    plus, minus = point.nuclei.positions.clone(), point.nuclei.positions.clone()
    plus[1, 2] += d
    minus[1, 2] -= d
    return (float(bo(plus, point.nuclei.charges, orb, *args))
            - float(bo(minus, point.nuclei.charges, orb, *args))) / (2 * d)


# ---- LiH ------------------------------------------------------------------------------

def test_lih_single_point_is_bound():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.lih import lih_hgh_elements, lih_initial_geometry, solve_rhf_at_geometry
    p = solve_rhf_at_geometry(lih_initial_geometry(3.0), lih_hgh_elements(), Grid3D(40, 12.0), max_iters=40,
                              mixing=0.5, order=4)
    assert p.converged and -2.0 < p.energy < -0.50, p.energy


def test_lih_first_iteration_vs_oracle():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.lih import lih_hgh_elements, lih_initial_geometry, solve_rhf_at_geometry
    nuc = lih_initial_geometry(3.1)
    onuc = o.Nuclei(nuc.positions.numpy(), nuc.charges.numpy())
    ref = o.solve_rhf_at_geometry(onuc, (o.lookup("Li"), o.lookup("H")), o.Grid3D(32, 12.0), max_iters=1,
                                  lanczos_iters=48)
    got = solve_rhf_at_geometry(nuc, lih_hgh_elements(), Grid3D(32, 12.0), max_iters=1, lanczos_iters=48)
    assert abs(got.energy - ref.energy) < 1e-10, (got.energy, ref.energy)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lih_hellmann_feynman_matches_finite_difference(precision):
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.lih import (bo_energy, bo_grad_positions, lih_hgh_elements, lih_initial_geometry,
                                        solve_rhf_at_geometry)
    g, el = Grid3D(28, 12.0), lih_hgh_elements()
    p = solve_rhf_at_geometry(lih_initial_geometry(3.1), el, g, max_iters=30, mixing=0.5, precision=precision)
    ga = bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, el, g, 4)
    assert float(ga[1, 2]) == pytest.approx(_fd_z(bo_energy, p, el, g, 4), rel=1e-3, abs=1e-4)


def test_lih_geometry_opt_recovers_bond_length():
    from gato_gb300.geometry import bond_length
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.lih import lih_hgh_elements, lih_initial_geometry, optimize_geometry
    res = optimize_geometry(lih_initial_geometry(3.8), lih_hgh_elements(), Grid3D(32, 12.0), geom_steps=15,
                            learning_rate=0.05, scf_max_iters=30, scf_mixing=0.5, order=4, verbose=False)
    R = float(bond_length(res.final.nuclei, 0, 1))
    assert 2.5 <= R <= 3.6 and abs(R - 3.8) > 0.1, R


# ---- HCl ------------------------------------------------------------------------------

def test_hcl_single_point_is_bound():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.hcl import hcl_hgh_elements, hcl_initial_geometry, solve_rhf_at_geometry
    p = solve_rhf_at_geometry(hcl_initial_geometry(2.4), hcl_hgh_elements(), Grid3D(24, 12.0), max_iters=60,
                              mixing=0.4, order=4)
    assert -20.0 < p.energy < -10.0, p.energy
    assert p.orbital_energies.shape == (4,) and all(float(e) < 0 for e in p.orbital_energies)


def test_hcl_first_iteration_vs_oracle():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.hcl import hcl_hgh_elements, hcl_initial_geometry, solve_rhf_at_geometry
    nuc = hcl_initial_geometry(2.4)
    onuc = o.Nuclei(nuc.positions.numpy(), nuc.charges.numpy())
    ref = o.solve_rhf_at_geometry(onuc, (o.lookup("H"), o.lookup("Cl")), o.Grid3D(32, 12.0), max_iters=1,
                                  lanczos_iters=60)
    got = solve_rhf_at_geometry(nuc, hcl_hgh_elements(), Grid3D(32, 12.0), max_iters=1, lanczos_iters=60)
    assert abs(got.energy - ref.energy) < 1e-10, (got.energy, ref.energy)
    assert np.max(np.abs(got.orbital_energies.cpu().numpy() - ref.orbital_energies)) < 1e-10


def test_hcl_nonlocal_apply_vs_oracle():
    """Cl drives the two-projector s channel with its off-diagonal h_12 (hcl.py:1-20)."""
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.hcl import hcl_hgh_elements, hcl_initial_geometry
    from gato_gb300.pseudopotentials import hgh_nonlocal_apply
    nuc = hcl_initial_geometry(2.4)
    onuc = o.Nuclei(nuc.positions.numpy(), nuc.charges.numpy())
    og = o.Grid3D(32, 12.0)
    psi = np.random.default_rng(5).standard_normal(og.shape)
    ref = o.hgh_nonlocal_apply(psi, onuc, (o.lookup("H"), o.lookup("Cl")), og)
    got = hgh_nonlocal_apply(torch.tensor(psi, device="cuda"), nuc, hcl_hgh_elements(), Grid3D(32, 12.0))
    assert np.max(np.abs(got.cpu().numpy() - ref)) < 1e-11 * max(1.0, np.max(np.abs(ref)))


def test_hcl_hellmann_feynman_matches_finite_difference():
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.hcl import (bo_energy, bo_grad_positions, hcl_hgh_elements, hcl_initial_geometry,
                                        solve_rhf_at_geometry)
    g, el = Grid3D(24, 12.0), hcl_hgh_elements()
    p = solve_rhf_at_geometry(hcl_initial_geometry(2.4), el, g, max_iters=60, mixing=0.4)
    ga = bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, el, g, 4)
    assert float(ga[1, 2]) == pytest.approx(_fd_z(bo_energy, p, el, g, 4), rel=1e-3, abs=1e-4)


def test_hcl_geometry_opt_moves_toward_equilibrium():
    from gato_gb300.geometry import bond_length
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.hcl import hcl_hgh_elements, hcl_initial_geometry, optimize_geometry
    res = optimize_geometry(hcl_initial_geometry(3.0), hcl_hgh_elements(), Grid3D(24, 12.0), geom_steps=10,
                            learning_rate=0.05, scf_max_iters=40, scf_mixing=0.4, order=4, verbose=False)
    R = float(bond_length(res.final.nuclei, 0, 1))
    assert 1.8 <= R <= 3.0 and R < 3.0 - 0.05, R


# ---- H2 -------------------------------------------------------------------------------

def test_h2_single_point_is_bound():
    from gato_gb300.geometry import diatomic_along_z
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.h2 import solve_rhf_at_geometry
    p = solve_rhf_at_geometry(diatomic_along_z(1.4, Z1=1.0), Grid3D(40, 10.0), max_iters=30, mixing=0.7)
    assert p.converged and -1.30 < p.energy < -1.0, p.energy


def test_h2_first_iteration_vs_oracle():
    from gato_gb300.geometry import diatomic_along_z
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.h2 import solve_rhf_at_geometry
    nuc = diatomic_along_z(1.5, Z1=1.0)
    og = o.Grid3D(32, 10.0)
    onuc = o.Nuclei(nuc.positions.numpy(), nuc.charges.numpy())
    eps = og.h / 2
    ref = o.scf_rhf(o.multi_center_softened_coulomb(onuc, og, eps), og, 1, max_iters=1, mixing=0.7,
                    epsilon=eps, lanczos_iters=48)
    got = solve_rhf_at_geometry(nuc, Grid3D(32, 10.0), max_iters=1, lanczos_iters=48)
    assert abs(got.rhf_energy - ref.energy) < 1e-10, (got.rhf_energy, ref.energy)


def test_softened_coulomb_grad_vs_oracle():
    from gato_gb300.geometry import Nuclei
    from gato_gb300.grid import Grid3D
    from gato_gb300.potentials import multi_center_softened_coulomb_grad
    og = o.Grid3D(40, 10.0)
    pos = np.array([[0.1, -0.2, -0.7], [0.0, 0.3, 0.75]])
    Z = np.array([1.0, 2.0])
    X, Y, Zc = og.coords()
    rho = np.exp(-0.5 * (X * X + Y * Y + Zc * Zc)) * (1.0 + 0.1 * X)
    ref = o.multi_center_softened_coulomb_grad(o.Nuclei(pos, Z), og, rho, 0.2)
    nuc = Nuclei(torch.tensor(pos), torch.tensor(Z))
    for dt, tol in ((torch.float64, 1e-11), (torch.float32, 1e-6)):
        got = multi_center_softened_coulomb_grad(nuc, Grid3D(40, 10.0), torch.tensor(rho, device="cuda", dtype=dt),
                                                 0.2).numpy()
        assert np.max(np.abs(got - ref)) < tol * np.max(np.abs(ref)), (dt, got, ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_h2_hellmann_feynman_matches_finite_difference(precision):
    from gato_gb300.geometry import diatomic_along_z
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.h2 import bo_energy, bo_grad_positions, solve_rhf_at_geometry
    g = Grid3D(28, 10.0)
    p = solve_rhf_at_geometry(diatomic_along_z(1.6, Z1=1.0), g, max_iters=20, mixing=0.7, precision=precision)
    eps = g.h / 2
    ga = bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, g, eps, 4)
    assert float(ga[1, 2]) == pytest.approx(_fd_z(bo_energy, p, g, eps, 4), rel=1e-3, abs=1e-4)


def test_h2_geometry_opt_recovers_bond_length():
    from gato_gb300.geometry import bond_length, diatomic_along_z
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.h2 import optimize_geometry
    res = optimize_geometry(diatomic_along_z(1.9, Z1=1.0), Grid3D(32, 10.0), geom_steps=15, learning_rate=0.05,
                            scf_max_iters=20, scf_mixing=0.7, order=4, verbose=False)
    R = float(bond_length(res.final.nuclei, 0, 1))
    assert 1.2 <= R <= 1.7 and abs(R - 1.9) > 0.1 and res.final.energy < -1.0, (R, res.final.energy)


# ---- helium ---------------------------------------------------------------------------

def test_helium_matches_oracle_and_virial():
    from gato_gb300.physics.helium import solve_helium
    og = o.Grid3D(32, 8.0)
    ref = o.scf_rhf(o.softened_coulomb(og, 2.0, og.h / 2), og, 1, max_iters=30, tol=1e-8, mixing=0.7)
    he = solve_helium(N=32, L=8.0, tol=1e-8, verbose=False)
    assert he.converged
    assert abs(he.energy - ref.energy) < 1e-8, (he.energy, ref.energy)
    assert abs(he.kinetic + he.potential + he.hartree + he.exchange - he.energy) < 1e-10
    assert 0.8 < he.virial_ratio < 1.2


@pytest.mark.parametrize("study", ["spacing", "box"])
def test_grid_convergence_sweeps(study, tmp_path):
    import json

    from gato_gb300.benchmarks.grid_convergence import main
    out_file = tmp_path / "conv.json"
    if study == "spacing":
        doc = main(["water", "spacing", "--N", "24", "32", "40", "--L", "10", "--precision", "mixed",
                    "--max-scf", "60", "--out", str(out_file), "--quiet"])
        fit = doc["summary"]["E_vs_h"]
    else:
        doc = main(["hcl", "box", "--sides", "8", "9", "10", "--h", "0.25", "--precision", "fp64",
                    "--max-scf", "60", "--out", str(out_file), "--quiet"])
        assert doc["summary"]["h_spread"] == 0.0 and [r["N"] for r in doc["records"]] == [32, 36, 40]
        fit = doc["summary"]["E_vs_inv_L"]
    assert all(r["converged"] for r in doc["records"])
    assert fit is not None and math_isfinite(fit["y_inf"])
    assert json.loads(out_file.read_text())["records"][0]["N"] == doc["records"][0]["N"]


def math_isfinite(x):
    import math
    return math.isfinite(x)
