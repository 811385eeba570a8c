"""Lithium hydride LiH: closed-shell RHF with HGH pseudopotentials (reference: physics/lih.py:1-311).

Li (Z_ion = 1, one s and three p projectors) and H, two valence electrons,
one doubly occupied sigma orbital. Same machinery as water: the HGH local
and non-local device operators, the SCF of ``scf.py``, and the hand-written
adjoint for the Hellmann-Feynman forces.
"""
from __future__ import annotations

from dataclasses import dataclass

from ..geometry import Nuclei, diatomic_along_z
from ..grid import Grid3D
from ..pseudopotentials import HGHParams, lookup
from ._diatomic import optimize_diatomic
from ._molecule import HGHModel, MoleculePoint, bo_energy_model, bo_grad_model, solve_closed_shell


def lih_initial_geometry(R_LiH: float = 3.3) -> Nuclei:
    """Li at -R/2, H at +R/2 along z (lih.py:61-65)."""
    return diatomic_along_z(R_LiH, Z1=3.0, Z2=1.0)


def lih_hgh_elements() -> tuple[HGHParams, ...]:
    """HGH parameters aligned with ``lih_initial_geometry`` (lih.py:68-70)."""
    return (lookup("Li"), lookup("H"))


def pp_nuclear_repulsion(nuclei: Nuclei, elements):
    """Sum_{i<j} Z_ion_i Z_ion_j / R_ij (lih.py:78-95)."""
    return HGHModel(elements).e_nn(nuclei)


@dataclass
class LiHPoint(MoleculePoint):
    """lih.py:103-113."""


def solve_rhf_at_geometry(nuclei: Nuclei, elements, grid: Grid3D, *, max_iters: int = 50, tol: float = 1e-6,
                          mixing: float = 0.5, order: int = 4, lanczos_iters: int | None = None,
                          initial_orbitals=None, precision: str = "fp64") -> LiHPoint:
    """RHF on a fixed nuclear configuration with HGH pseudopotentials (lih.py:116-150)."""
    return solve_closed_shell(HGHModel(elements), nuclei, grid, max_iters=max_iters, tol=tol, mixing=mixing,
                              order=order, lanczos_iters=lanczos_iters, initial_orbitals=initial_orbitals,
                              precision=precision, point_cls=LiHPoint)


def bo_energy(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4):
    """Total BO energy at fixed orbitals, differentiable in positions (lih.py:158-176)."""
    return bo_energy_model(HGHModel(elements), positions, charges, orbitals, grid, order)


def bo_grad_positions(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4):
    """dE/dR at fixed orbitals (lih.py:181-187)."""
    return bo_grad_model(HGHModel(elements), positions, charges, orbitals, grid, order)


def hellmann_feynman_force(point: LiHPoint, elements, grid: Grid3D, order: int = 4):
    """-dE/dR at the converged orbitals, (2, 3)."""
    return -bo_grad_positions(point.nuclei.positions, point.nuclei.charges, point.orbitals, elements, grid,
                              order)


@dataclass
class LiHGeomOptResult:
    final: LiHPoint
    trajectory: list   # (step, energy, R_LiH)


def optimize_geometry(initial_nuclei: Nuclei, elements, grid: Grid3D, *, geom_steps: int = 30,
                      learning_rate: float = 0.05, scf_max_iters: int = 50, scf_tol: float = 1e-6,
                      scf_mixing: float = 0.5, order: int = 4, verbose: bool = True,
                      precision: str = "fp64") -> LiHGeomOptResult:
    """Alternating SCF + Adam on positions (lih.py:198-266)."""
    def solve_at(nuclei, prev):
        return solve_rhf_at_geometry(nuclei, elements, grid, initial_orbitals=prev.orbitals if prev else None,
                                     max_iters=scf_max_iters, tol=scf_tol, mixing=scf_mixing, order=order,
                                     precision=precision)

    def bo_grad(p):
        return bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, elements, grid, order)

    final, traj = optimize_diatomic(initial_nuclei, solve_at, bo_grad, geom_steps=geom_steps,
                                    learning_rate=learning_rate, label="R_LiH", verbose=verbose)
    return LiHGeomOptResult(final, traj)
