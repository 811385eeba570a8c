"""Closed-shell molecule machinery shared by the physics drivers.

The reference repeats the same three pieces in every molecule module
(physics/water.py:129-241, physics/lih.py:103-187, physics/hcl.py:135-219,
physics/h2.py:67-135): an RHF solve at fixed nuclei, the Born-Oppenheimer
energy at fixed orbitals, and its position gradient through jax.grad. Here
they are written once against a potential model, which says how V_ext, the
non-local part, the Coulomb softening and the nuclear repulsion depend on
the nuclei:

* ``HGHModel``: HGH local + separable non-local pseudopotentials, E_nn with
  the valence charges Z_ion, the Hartree/exchange kernel softened by h/2
  (water, LiH, HCl);
* ``SoftCoulombModel``: the multi-centre softened Coulomb V_ext, bare E_nn,
  one softening eps for V_ext and the Hartree/exchange kernel (H2).

``BOEnergy`` is a torch.autograd.Function whose backward is the
hand-written adjoint: d/dR of int rho V_ext (a device reduction per model),
the projector-overlap derivatives of V_nl, dE_nn/dR, and dE/dphi_i =
4 F phi_i dV for the orbitals.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from ..geometry import Nuclei, _t, nuclear_repulsion
from ..grid import Grid3D
from ..potentials import multi_center_softened_coulomb, multi_center_softened_coulomb_grad
from ..pseudopotentials import hgh_local_grad, hgh_local_potential, nonlocal_for, total_valence_charge
from ..scf import Operator, _density_fields, _energy_terms, pair_fields, precision_dtype, scf_rhf, to_fields
from ..solvers.poisson import get_plan


def _coulomb_pair_grad(pos: torch.Tensor, Z) -> torch.Tensor:
    """d/dR of sum_{i<j} Z_i Z_j / |R_i - R_j|, (K, 3)."""
    g = torch.zeros_like(pos)
    for a in range(pos.shape[0]):
        for b in range(pos.shape[0]):
            if a != b:
                d = pos[a] - pos[b]
                g[a] -= Z[a] * Z[b] * d / torch.linalg.norm(d) ** 3
    return g


class HGHModel:
    """HGH pseudopotential ions (pseudopotentials.py:201-405)."""

    def __init__(self, elements):
        self.elements = tuple(elements)

    def n_electrons(self, nuclei: Nuclei) -> int:
        return int(total_valence_charge(self.elements))

    def epsilon(self, grid: Grid3D) -> float:
        return grid.h / 2

    def v_ext(self, nuclei: Nuclei, grid: Grid3D, dtype) -> torch.Tensor:
        return hgh_local_potential(nuclei, self.elements, grid, dtype)

    def nonlocal_op(self, nuclei: Nuclei, grid: Grid3D, dtype):
        return nonlocal_for(nuclei, self.elements, grid, dtype)

    def v_ext_grad(self, nuclei: Nuclei, grid: Grid3D, rho) -> torch.Tensor:
        return hgh_local_grad(nuclei, self.elements, grid, rho)

    def _zion(self):
        return torch.tensor([p.Z_ion for p in self.elements], dtype=torch.float64)

    def e_nn(self, nuclei: Nuclei) -> torch.Tensor:
        """Sum_{i<j} Z_ion_i Z_ion_j / R_ij (water.py:100-110)."""
        return nuclear_repulsion(Nuclei(_t(nuclei.positions), self._zion()))

    def e_nn_grad(self, nuclei: Nuclei) -> torch.Tensor:
        return _coulomb_pair_grad(_t(nuclei.positions).detach().to(torch.float64), self._zion().tolist())


class SoftCoulombModel:
    """All-electron nuclei with the softened Coulomb potential (potentials.py:39-61)."""

    def __init__(self, epsilon: float | None = None):
        self.eps = epsilon

    def n_electrons(self, nuclei: Nuclei) -> int:
        return int(round(float(_t(nuclei.charges).sum())))

    def epsilon(self, grid: Grid3D) -> float:
        return grid.h / 2 if self.eps is None else float(self.eps)

    def v_ext(self, nuclei: Nuclei, grid: Grid3D, dtype) -> torch.Tensor:
        return multi_center_softened_coulomb(nuclei, grid, self.epsilon(grid), dtype=dtype)

    def nonlocal_op(self, nuclei: Nuclei, grid: Grid3D, dtype):
        return None

    def v_ext_grad(self, nuclei: Nuclei, grid: Grid3D, rho) -> torch.Tensor:
        return multi_center_softened_coulomb_grad(nuclei, grid, rho, self.epsilon(grid))

    def e_nn(self, nuclei: Nuclei) -> torch.Tensor:
        return nuclear_repulsion(Nuclei(_t(nuclei.positions), _t(nuclei.charges)))

    def e_nn_grad(self, nuclei: Nuclei) -> torch.Tensor:
        return _coulomb_pair_grad(_t(nuclei.positions).detach().to(torch.float64),
                                  _t(nuclei.charges).to(torch.float64).tolist())


@dataclass
class MoleculePoint:
    """One converged geometry: the fields of the reference's WaterPoint / LiHPoint / HClPoint / H2Point."""

    nuclei: Nuclei
    orbitals: torch.Tensor
    energy: float                # E_RHF + E_nn
    rhf_energy: float
    nuclear_repulsion: float
    n_iters: int
    converged: bool
    orbital_energies: torch.Tensor


def solve_closed_shell(model, nuclei: Nuclei, grid: Grid3D, *, n_occ: int | None = None, max_iters: int,
                       tol: float, mixing: float, order: int, lanczos_iters: int | None,
                       initial_orbitals, precision: str, point_cls=MoleculePoint):
    """scf_rhf at fixed nuclei plus E_nn (water.py:129-174, lih.py:103-150, h2.py:67-100)."""
    dtype = precision_dtype(precision)
    if n_occ is None:
        n_electrons = model.n_electrons(nuclei)
        if n_electrons % 2 != 0:
            raise ValueError(f"Closed-shell RHF requires even electron count; got {n_electrons}")
        n_occ = n_electrons // 2
    # V_ext stays FP64: the SCF evaluates the energy in FP64 under either precision
    V_ext = model.v_ext(nuclei, grid, torch.float64)
    res = scf_rhf(V_ext, grid, n_occ=n_occ, initial_orbitals=initial_orbitals, max_iters=max_iters, tol=tol,
                  mixing=mixing, order=order, lanczos_iters=lanczos_iters, epsilon=model.epsilon(grid),
                  V_nl_apply=model.nonlocal_op(nuclei, grid, dtype), precision=precision)
    E_nn = float(model.e_nn(nuclei))
    return point_cls(nuclei, res.orbitals, float(res.energy) + E_nn, float(res.energy), E_nn, res.n_iters,
                     res.converged, res.orbital_energies)


class BOEnergy(torch.autograd.Function):
    """E(R, phi) = E_RHF[phi; V_ext(R), V_nl(R)] + E_nn(R) with a hand-written adjoint."""

    @staticmethod
    def forward(ctx, positions, fields, charges, model, grid, order):
        nuclei = Nuclei(positions.detach().to(torch.float64).cpu(), charges)
        dtype = fields.dtype
        eps = model.epsilon(grid)
        V_ext = model.v_ext(nuclei, grid, dtype)
        nl = model.nonlocal_op(nuclei, grid, dtype)
        terms = _energy_terms(fields, V_ext, grid, "dirichlet", order, eps, nl)
        E = terms.sum().cpu() + model.e_nn(nuclei).detach()
        ctx.save_for_backward(fields)
        ctx.nuclei, ctx.model, ctx.grid, ctx.order = nuclei, model, grid, order
        ctx.V_ext, ctx.nl = V_ext, nl
        return E.to(positions.dtype)

    @staticmethod
    def backward(ctx, gE):
        (fields,) = ctx.saved_tensors
        nuclei, model, grid = ctx.nuclei, ctx.model, ctx.grid
        g_pos = g_fields = None
        if ctx.needs_input_grad[0]:
            g = model.v_ext_grad(nuclei, grid, _density_fields(fields))
            if ctx.nl is not None:
                g = g + ctx.nl.grad(fields)
            g = g + model.e_nn_grad(nuclei)
            g_pos = gE.cpu().to(torch.float64) * g
        if ctx.needs_input_grad[1]:
            # dE/dphi_i(r) = 4 (F phi_i)(r) dV, F built from these orbitals
            dtype = fields.dtype
            plan = get_plan(grid.N, grid.h, model.epsilon(grid), dtype, pair_fields(fields.shape[0]))
            op = Operator(grid, dtype, ctx.order, "dirichlet")
            V_tot = ctx.V_ext + plan.potential(_density_fields(fields))
            op.set_potential(V_tot.contiguous())
            op.set_nonlocal(ctx.nl)
            op.set_exchange(plan, fields)
            g_fields = op.apply_block() * (4.0 * grid.dV) * gE.to(fields.device, fields.dtype)
        return g_pos, g_fields, None, None, None, None


def bo_energy_model(model, positions, charges, orbitals, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """Total BO energy at fixed orbitals, differentiable in positions (and in the orbitals)."""
    return BOEnergy.apply(_t(positions), to_fields(orbitals), _t(charges), model, grid, order)


def bo_grad_model(model, positions, charges, orbitals, grid: Grid3D, order: int = 4) -> torch.Tensor:
    """dE/dR at fixed orbitals (jax.grad of the BO energy in the reference): the adjoint kernels alone.

    The position gradient of BOEnergy is its backward with dE/dE = 1, and it needs none of the
    forward's energy terms (the kinetic, Hartree and exchange terms do not depend on R), so the
    energy pass is skipped. The sum runs in the backward's order, so the result is the same.
    ``order`` only enters the energy and is kept for the reference's signature."""
    p = _t(positions)
    fields = to_fields(orbitals)
    nuclei = Nuclei(p.detach().to(torch.float64).cpu(), _t(charges))
    g = model.v_ext_grad(nuclei, grid, _density_fields(fields))
    nl = model.nonlocal_op(nuclei, grid, fields.dtype)
    if nl is not None:
        g = g + nl.grad(fields)
    g = g + model.e_nn_grad(nuclei)
    return g.to(dtype=p.dtype, device=p.device)
