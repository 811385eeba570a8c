"""Helium-like atoms by closed-shell RHF (reference: physics/helium.py:1-170).

One doubly occupied orbital around a softened Coulomb nucleus of charge Z;
the same softening eps (default h/2) for V_ext and the Hartree/exchange
kernel. Reports the energy decomposition and the Coulomb virial ratio
2<T> / |<V_ext> + E_H + E_x|.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from ..grid import Grid3D
from ..potentials import softened_coulomb
from ..scf import _density, decompose_rhf_energy, scf_rhf


@dataclass
class HeliumResult:
    """helium.py:35-52."""

    grid: Grid3D
    orbitals: torch.Tensor          # (N, N, N, 1)
    psi: torch.Tensor               # (N, N, N)
    density: torch.Tensor           # rho = 2 |phi|^2
    V_ext: torch.Tensor
    energy: float
    kinetic: float                  # 2 sum_i <phi_i|T|phi_i>
    potential: float                # 2 sum_i <phi_i|V_ext|phi_i>
    hartree: float
    exchange: float
    virial_ratio: float             # 2<T> / |<V_ext> + E_H + E_x|
    orbital_energies: torch.Tensor
    n_iters: int
    converged: bool
    history: list


def solve_helium(N: int = 64, L: float = 10.0, Z: float = 2.0, epsilon: float | None = None,
                 max_iters: int = 30, tol: float = 1e-6, mixing: float = 0.7, order: int = 4,
                 lanczos_iters: int | None = None, verbose: bool = True, precision: str = "fp64",
                 initial_orbitals=None) -> HeliumResult:
    """Solve closed-shell helium (or He-like Z = 3, 4, ...) by RHF (helium.py:55-160)."""
    grid = Grid3D(N=N, L=L)
    V_ext = softened_coulomb(grid, Z=Z, epsilon=epsilon)
    result = scf_rhf(V_ext, grid, n_occ=1, initial_orbitals=initial_orbitals, max_iters=max_iters, tol=tol,
                     mixing=mixing, order=order, lanczos_iters=lanczos_iters, epsilon=epsilon,
                     precision=precision)
    orbitals = result.orbitals
    terms = decompose_rhf_energy(orbitals, V_ext, grid, boundary="dirichlet", order=order, epsilon=epsilon)
    T, V_exp = float(terms.kinetic), float(terms.v_ext)
    E_H, E_x = float(terms.hartree), float(terms.exchange)
    vr = 2.0 * T / abs(V_exp + E_H + E_x)
    out = HeliumResult(grid=grid, orbitals=orbitals, psi=orbitals[..., 0], density=_density(orbitals), V_ext=V_ext,
                       energy=float(result.energy), kinetic=T, potential=V_exp, hartree=E_H, exchange=E_x,
                       virial_ratio=vr, orbital_energies=result.orbital_energies, n_iters=result.n_iters,
                       converged=result.converged,
                       history=[(i + 1, e) for i, e in enumerate(result.energy_history)])
    if verbose:
        summary = {"E": out.energy, "T": T, "V_ext": V_exp, "E_H": E_H, "E_x": E_x,
                   "eps_1": float(result.orbital_energies[0]), "2T/|V|": vr}
        print(f"He-like Z={Z:g} N={N} L={L:g} order={order}: SCF {result.n_iters} iterations "
              f"(converged={result.converged}); " + ", ".join(f"{k}={v:.6f}" for k, v in summary.items()))
    return out
