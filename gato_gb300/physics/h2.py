"""H2 with closed-shell RHF and the softened Coulomb nuclei (reference: physics/h2.py:1-261).

No pseudopotentials: V_ext is the multi-centre softened Coulomb potential,
and the same softening eps (default h/2) is used for the Hartree/exchange
kernel. One doubly occupied sigma_g orbital. Forces come from the
hand-written adjoint (``BOEnergy``) with the device reduction
int rho dV_ext/dR for the softened Coulomb centres.
"""
from __future__ import annotations

from dataclasses import dataclass

from ..geometry import Nuclei, diatomic_along_z  # noqa: F401
from ..grid import Grid3D
from ._diatomic import optimize_diatomic
from ._molecule import MoleculePoint, SoftCoulombModel, bo_energy_model, bo_grad_model, solve_closed_shell


@dataclass
class H2Point(MoleculePoint):
    """h2.py:55-65."""


def solve_rhf_at_geometry(nuclei: Nuclei, grid: Grid3D, *, epsilon: float | None = None, max_iters: int = 30,
                          tol: float = 1e-6, mixing: float = 0.7, order: int = 4,
                          lanczos_iters: int | None = None, initial_orbitals=None,
                          precision: str = "fp64") -> H2Point:
    """RHF on a fixed nuclear configuration with bare (softened) Coulomb (h2.py:67-100)."""
    return solve_closed_shell(SoftCoulombModel(epsilon), nuclei, grid, n_occ=1, max_iters=max_iters, tol=tol,
                              mixing=mixing, order=order, lanczos_iters=lanczos_iters,
                              initial_orbitals=initial_orbitals, precision=precision, point_cls=H2Point)


def bo_energy(positions, charges, orbitals, grid: Grid3D, epsilon: float, order: int = 4):
    """Total BO energy at fixed orbitals, differentiable in positions (h2.py:107-128)."""
    return bo_energy_model(SoftCoulombModel(epsilon), positions, charges, orbitals, grid, order)


def bo_grad_positions(positions, charges, orbitals, grid: Grid3D, epsilon: float, order: int = 4):
    """dE/dR at fixed orbitals (h2.py:131-135)."""
    return bo_grad_model(SoftCoulombModel(epsilon), positions, charges, orbitals, grid, order)


def hellmann_feynman_force(point: H2Point, grid: Grid3D, epsilon: float | None = None, order: int = 4):
    """-dE/dR at the converged orbitals, (2, 3)."""
    eps = grid.h / 2 if epsilon is None else epsilon
    return -bo_grad_positions(point.nuclei.positions, point.nuclei.charges, point.orbitals, grid, eps, order)


@dataclass
class H2GeomOptResult:
    final: H2Point
    trajectory: list   # (step, energy, R_HH)


def optimize_geometry(initial_nuclei: Nuclei, grid: Grid3D, *, epsilon: float | None = None,
                      geom_steps: int = 30, learning_rate: float = 0.05, scf_max_iters: int = 30,
                      scf_tol: float = 1e-6, scf_mixing: float = 0.7, order: int = 4, verbose: bool = True,
                      precision: str = "fp64") -> H2GeomOptResult:
    """Alternating SCF + Adam on positions (h2.py:146-214)."""
    eps = grid.h / 2 if epsilon is None else epsilon

    def solve_at(nuclei, prev):
        return solve_rhf_at_geometry(nuclei, grid, epsilon=eps, initial_orbitals=prev.orbitals if prev else None,
                                     max_iters=scf_max_iters, tol=scf_tol, mixing=scf_mixing, order=order,
                                     precision=precision)

    def bo_grad(p):
        return bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, grid, eps, order)

    final, traj = optimize_diatomic(initial_nuclei, solve_at, bo_grad, geom_steps=geom_steps,
                                    learning_rate=learning_rate, label="R_HH", verbose=verbose)
    return H2GeomOptResult(final, traj)
