"""Hydrogen chloride HCl: closed-shell RHF with HGH pseudopotentials (reference: physics/hcl.py:1-351).

H and Cl (Z_ion = 7: two coupled s projectors with h_12 and three p projectors),
eight valence electrons, four doubly occupied orbitals. Same machinery as
water: the HGH local and non-local device operators, the SCF of ``scf.py``,
and the hand-written adjoint for the Hellmann-Feynman forces.
"""
from __future__ import annotations

from dataclasses import dataclass

from ..geometry import Nuclei, diatomic_along_z
from ..grid import Grid3D
from ..pseudopotentials import HGHParams, lookup
from ._diatomic import optimize_diatomic
from ._molecule import HGHModel, MoleculePoint, bo_energy_model, bo_grad_model, solve_closed_shell


def hcl_initial_geometry(R_HCl: float = 2.6) -> Nuclei:
    """H at -R/2, Cl at +R/2 along z (hcl.py:89-97)."""
    return diatomic_along_z(R_HCl, Z1=1.0, Z2=17.0)


def hcl_hgh_elements() -> tuple[HGHParams, ...]:
    """HGH parameters aligned with ``hcl_initial_geometry`` (hcl.py:100-102)."""
    return (lookup("H"), lookup("Cl"))


def pp_nuclear_repulsion(nuclei: Nuclei, elements):
    """Sum_{i<j} Z_ion_i Z_ion_j / R_ij (hcl.py:109-123)."""
    return HGHModel(elements).e_nn(nuclei)


@dataclass
class HClPoint(MoleculePoint):
    """hcl.py:130-139."""


def solve_rhf_at_geometry(nuclei: Nuclei, elements, grid: Grid3D, *, max_iters: int = 60, tol: float = 1e-6,
                          mixing: float = 0.5, order: int = 4, lanczos_iters: int | None = None,
                          initial_orbitals=None, precision: str = "fp64") -> HClPoint:
    """RHF on a fixed nuclear configuration with HGH pseudopotentials (hcl.py:142-185)."""
    return solve_closed_shell(HGHModel(elements), nuclei, grid, max_iters=max_iters, tol=tol, mixing=mixing,
                              order=order, lanczos_iters=lanczos_iters, initial_orbitals=initial_orbitals,
                              precision=precision, point_cls=HClPoint)


def bo_energy(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4):
    """Total BO energy at fixed orbitals, differentiable in positions (hcl.py:192-212)."""
    return bo_energy_model(HGHModel(elements), positions, charges, orbitals, grid, order)


def bo_grad_positions(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4):
    """dE/dR at fixed orbitals (hcl.py:215-221)."""
    return bo_grad_model(HGHModel(elements), positions, charges, orbitals, grid, order)


def hellmann_feynman_force(point: HClPoint, elements, grid: Grid3D, order: int = 4):
    """-dE/dR at the converged orbitals, (2, 3)."""
    return -bo_grad_positions(point.nuclei.positions, point.nuclei.charges, point.orbitals, elements, grid,
                              order)


@dataclass
class HClGeomOptResult:
    final: HClPoint
    trajectory: list   # (step, energy, R_HCl)


def optimize_geometry(initial_nuclei: Nuclei, elements, grid: Grid3D, *, geom_steps: int = 30,
                      learning_rate: float = 0.05, scf_max_iters: int = 60, scf_tol: float = 1e-6,
                      scf_mixing: float = 0.5, order: int = 4, verbose: bool = True,
                      precision: str = "fp64") -> HClGeomOptResult:
    """Alternating SCF + Adam on positions (hcl.py:234-283)."""
    def solve_at(nuclei, prev):
        return solve_rhf_at_geometry(nuclei, elements, grid, initial_orbitals=prev.orbitals if prev else None,
                                     max_iters=scf_max_iters, tol=scf_tol, mixing=scf_mixing, order=order,
                                     precision=precision)

    def bo_grad(p):
        return bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, elements, grid, order)

    final, traj = optimize_diatomic(initial_nuclei, solve_at, bo_grad, geom_steps=geom_steps,
                                    learning_rate=learning_rate, label="R_HCl", verbose=verbose)
    return HClGeomOptResult(final, traj)
