"""H2O with RHF + HGH pseudopotentials (reference: physics/water.py:1-392).

Forces: ``bo_energy`` is a torch.autograd.Function whose backward is the
hand-written adjoint: the Hellmann-Feynman derivative of the R-dependent
terms (int rho dV_loc/dR on the grid, the projector-overlap derivatives of
the non-local part, and dE_nn/dR), plus dE/dphi_i = 4 F phi_i dV for the
orbitals. The reference obtains the position gradient with jax.grad
(water.py:221-241).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from .. import _lib
from ..geometry import Nuclei, _t, bond_angle, bond_length, nuclear_repulsion
from ..geometry_opt import optimize_geometry_alternating
from ..grid import Grid3D, as_field
from ..pseudopotentials import (HGHParams, hgh_local_grad, hgh_local_potential, lookup,
                                nonlocal_for, total_valence_charge)
from ..scf import (Operator, _density_fields, _energy_terms, from_fields, pair_fields,
                   precision_dtype, scf_rhf, to_fields)
from ..solvers.poisson import get_plan


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
    return nuclear_repulsion(Nuclei(_t(nuclei.positions),
                                    torch.tensor([p.Z_ion for p in elements], dtype=torch.float64)))


def pp_nuclear_repulsion_grad(nuclei: Nuclei, elements) -> torch.Tensor:
    p = _t(nuclei.positions).detach().to(torch.float64)
    Z = [pe.Z_ion for pe in elements]
    g = torch.zeros_like(p)
    for a in range(p.shape[0]):
        for b in range(p.shape[0]):
            if a != b:
                d = p[a] - p[b]
                g[a] -= Z[a] * Z[b] * d / torch.linalg.norm(d) ** 3
    return g


@dataclass
class WaterPoint:
    nuclei: Nuclei
    orbitals: torch.Tensor
    energy: float
    rhf_energy: float
    nuclear_repulsion: float
    n_iters: int
    converged: bool
    orbital_energies: torch.Tensor


def solve_rhf_at_geometry(nuclei: Nuclei, elements, grid: Grid3D, *, max_iters: int = 60, tol: float = 1e-6,
                          mixing: float = 0.5, order: int = 4, lanczos_iters: int | None = None,
                          initial_orbitals=None, precision: str = "fp64") -> WaterPoint:
    """RHF on a fixed geometry with HGH pseudopotentials (water.py:129-174)."""
    dtype = precision_dtype(precision)
    # V_loc stays FP64: the SCF evaluates the energy in FP64 under either precision
    V_local = hgh_local_potential(nuclei, elements, grid, torch.float64)
    V_nl = nonlocal_for(nuclei, elements, grid, dtype)
    n_electrons = int(total_valence_charge(elements))
    if n_electrons % 2 != 0:
        raise ValueError(f"Closed-shell RHF requires even electron count; got {n_electrons}")
    res = scf_rhf(V_local, grid, n_occ=n_electrons // 2, initial_orbitals=initial_orbitals,
                  max_iters=max_iters, tol=tol, mixing=mixing, order=order, lanczos_iters=lanczos_iters,
                  V_nl_apply=V_nl, precision=precision)
    E_nn = float(pp_nuclear_repulsion(nuclei, elements))
    return WaterPoint(nuclei, res.orbitals, float(res.energy) + E_nn, float(res.energy), E_nn, res.n_iters,
                      res.converged, res.orbital_energies)


class BOEnergy(torch.autograd.Function):
    """E(R, phi) = E_RHF[phi; V_loc(R), V_nl(R)] + E_nn(R) with a hand-written adjoint."""

    @staticmethod
    def forward(ctx, positions, fields, charges, elements, grid, order):
        nuclei = Nuclei(positions.detach().to(torch.float64).cpu(), charges)
        dtype = fields.dtype
        V_local = hgh_local_potential(nuclei, elements, grid, dtype)
        nl = nonlocal_for(nuclei, elements, grid, dtype)
        terms = _energy_terms(fields, V_local, grid, "dirichlet", order, grid.h / 2, nl)
        E = terms.sum().cpu() + pp_nuclear_repulsion(nuclei, elements).detach()
        ctx.save_for_backward(fields)
        ctx.nuclei, ctx.elements, ctx.grid, ctx.order = nuclei, elements, grid, order
        ctx.V_local, ctx.nl = V_local, nl
        return E.to(positions.dtype)

    @staticmethod
    def backward(ctx, gE):
        (fields,) = ctx.saved_tensors
        nuclei, elements, grid = ctx.nuclei, ctx.elements, ctx.grid
        g_pos = g_fields = None
        if ctx.needs_input_grad[0]:
            rho = _density_fields(fields)
            g = hgh_local_grad(nuclei, elements, grid, rho)
            g = g + ctx.nl.grad(fields)
            g = g + pp_nuclear_repulsion_grad(nuclei, elements)
            g_pos = gE.cpu().to(torch.float64) * g
        if ctx.needs_input_grad[1]:
            # dE/dphi_i(r) = 4 (F phi_i)(r) dV, F built from these orbitals
            dtype = fields.dtype
            eps = grid.h / 2
            plan = get_plan(grid.N, grid.h, eps, dtype, pair_fields(fields.shape[0]))
            op = Operator(grid, dtype, ctx.order, "dirichlet")
            V_tot = ctx.V_local + plan.potential(_density_fields(fields))
            op.set_potential(V_tot.contiguous())
            op.set_nonlocal(ctx.nl)
            op.set_exchange(plan, fields)
            g_fields = op.apply_block() * (4.0 * grid.dV) * gE.to(fields.device, fields.dtype)
        return g_pos, g_fields, None, None, None, None


def bo_energy(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """Total BO energy at fixed orbitals (water.py:181-215), differentiable in positions."""
    positions = _t(positions)
    fields = to_fields(orbitals)
    return BOEnergy.apply(positions, fields, _t(charges), tuple(elements), grid, order)


def bo_grad_positions(positions, charges, orbitals, elements, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """dE/dR at fixed orbitals: the adjoint kernels alone (water.py:221-224)."""
    p = _t(positions).detach().clone().requires_grad_(True)
    E = bo_energy(p, charges, orbitals, elements, grid, order)
    (g,) = torch.autograd.grad(E, p)
    return g


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
