"""H2O with RHF + HGH pseudopotentials (reference: physics/water.py:1-392).

Forces: ``bo_energy`` goes through ``BOEnergy`` (physics/_molecule.py), a
torch.autograd.Function whose backward is the hand-written adjoint: the
Hellmann-Feynman derivative of the R-dependent terms (int rho dV_loc/dR on
the grid, the projector-overlap derivatives of the non-local part, and
dE_nn/dR), plus dE/dphi_i = 4 F phi_i dV for the orbitals. The reference
obtains the position gradient with jax.grad (water.py:221-241).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from ..geometry import Nuclei, bond_angle, bond_length
from ..geometry_opt import optimize_geometry_alternating
from ..grid import Grid3D
from ..pseudopotentials import HGHParams, lookup
from ._molecule import (BOEnergy, HGHModel, MoleculePoint, bo_energy_model, bo_grad_model,  # noqa: F401
                        solve_closed_shell)


def water_initial_geometry(R_OH: float = 1.85, angle_deg: float = 100.0) -> Nuclei:
    """O at the origin, both H in the xz-plane at +-half angle (water.py:66-82)."""
    half = math.radians(angle_deg) / 2.0
    pos = torch.tensor([[0.0, 0.0, 0.0],
                        [R_OH * math.sin(half), 0.0, R_OH * math.cos(half)],
                        [-R_OH * math.sin(half), 0.0, R_OH * math.cos(half)]], dtype=torch.float64)
    return Nuclei(pos, torch.tensor([8.0, 1.0, 1.0], dtype=torch.float64))


def water_hgh_elements() -> tuple[HGHParams, ...]:
    return (lookup("O"), lookup("H"), lookup("H"))


def pp_nuclear_repulsion(nuclei: Nuclei, elements) -> torch.Tensor:
    """E_nn with the valence charges Z_ion (water.py:100-110)."""
    return HGHModel(elements).e_nn(nuclei)


def pp_nuclear_repulsion_grad(nuclei: Nuclei, elements) -> torch.Tensor:
    return HGHModel(elements).e_nn_grad(nuclei)


@dataclass
class WaterPoint(MoleculePoint):
    """nuclei, orbitals, energy (E_RHF + E_nn), rhf_energy, nuclear_repulsion, n_iters, converged,
    orbital_energies (water.py:113-126)."""


def solve_rhf_at_geometry(nuclei: Nuclei, elements, grid: Grid3D, *, max_iters: int = 60, tol: float = 1e-6,
                          mixing: float = 0.5, order: int = 4, lanczos_iters: int | None = None,
                          initial_orbitals=None, precision: str = "fp64") -> WaterPoint:
    """RHF on a fixed geometry with HGH pseudopotentials (water.py:129-174)."""
    return solve_closed_shell(HGHModel(elements), nuclei, grid, max_iters=max_iters, tol=tol, mixing=mixing,
                              order=order, lanczos_iters=lanczos_iters, initial_orbitals=initial_orbitals,
                              precision=precision, point_cls=WaterPoint)


def bo_energy(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """Total BO energy at fixed orbitals (water.py:181-215), differentiable in positions."""
    return bo_energy_model(HGHModel(elements), positions, charges, orbitals, grid, order)


def bo_grad_positions(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """dE/dR at fixed orbitals: the adjoint kernels alone (water.py:221-224)."""
    return bo_grad_model(HGHModel(elements), positions, charges, orbitals, grid, order)


def hellmann_feynman_force(point: WaterPoint, elements, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """Force on every nucleus, (K, 3); valid at converged orbitals (water.py:227-241)."""
    return -bo_grad_positions(point.nuclei.positions, point.nuclei.charges, point.orbitals, elements, grid,
                              order)


@dataclass
class WaterGeomOptResult:
    final: WaterPoint
    trajectory: list


def optimize_water_geometry(initial_nuclei: Nuclei, elements, grid: Grid3D, *, geom_steps: int = 30,
                            learning_rate: float = 0.05, scf_max_iters: int = 60, scf_tol: float = 1e-6,
                            scf_mixing: float = 0.5, order: int = 4, lanczos_iters: int | None = None,
                            verbose: bool = True, precision: str = "fp64") -> WaterGeomOptResult:
    """Alternating SCF + Adam on the Hellmann-Feynman gradient (water.py:254-318)."""

    def solve_at(nuclei, prev):
        return solve_rhf_at_geometry(nuclei, elements, grid, initial_orbitals=prev.orbitals if prev else None,
                                     max_iters=scf_max_iters, tol=scf_tol, mixing=scf_mixing, order=order,
                                     lanczos_iters=lanczos_iters, precision=precision)

    def bo_grad(p):
        return bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, elements, grid, order)

    trajectory = []

    def on_step(step, p):
        R = float(bond_length(p.nuclei, 0, 1))
        ang = math.degrees(float(bond_angle(p.nuclei, 1, 0, 2)))
        trajectory.append((step, p.energy, R, ang))
        if verbose:
            print(f"  geom step {step:3d}  E = {p.energy:+.6f}  R_OH = {R:.4f} a0  angle = {ang:.2f} deg  "
                  f"SCF iters = {p.n_iters}")

    final, _ = optimize_geometry_alternating(initial_nuclei, solve_at_geometry=solve_at, bo_grad=bo_grad,
                                             geom_steps=geom_steps, learning_rate=learning_rate,
                                             on_step=on_step)
    return WaterGeomOptResult(final, trajectory)
