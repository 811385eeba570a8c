"""Hydrogen-like atom by imaginary-time propagation (reference: physics/hydrogen.py:1-133).

One electron in a softened Coulomb well of charge Z; the ground state from
``imaginary_time`` (a CUDA-graph replayed Euler step), then the observables
<T>, <V> and the virial ratio. E_0(Z) = -Z^2 / 2 Ha analytically.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from ..ansatz import init_grid_ansatz
from ..grid import Grid3D, normalize
from ..hamiltonian import Hamiltonian
from ..observables import kinetic_energy, potential_energy, virial_ratio
from ..potentials import softened_coulomb
from ..solvers.imag_time import imaginary_time


@dataclass
class HydrogenResult:
    """hydrogen.py:27-36."""

    grid: Grid3D
    psi: torch.Tensor
    V: torch.Tensor
    energy: float
    kinetic: float
    potential: float
    virial_ratio: float
    history: list


def solve_hydrogen(N: int = 48, L: float = 10.0, Z: float = 1.0, epsilon: float | None = None,
                   n_steps: int = 3000, order: int = 2, seed: int = 0, verbose: bool = True) -> HydrogenResult:
    """Hydrogen-like ground state for nuclear charge Z at the origin (hydrogen.py:39-102)."""
    grid = Grid3D(N=N, L=L)
    V = softened_coulomb(grid, Z=Z, epsilon=epsilon)
    H = Hamiltonian(grid=grid, V=V, boundary="dirichlet", order=order)
    psi0 = init_grid_ansatz(grid, seed, init="hydrogenic", Z=Z)
    psi, history = imaginary_time(H, psi0, n_steps=n_steps, log_every=max(1, n_steps // 20))
    hist = list(zip(history.steps, history.energies))
    psi = normalize(psi, grid)
    T = float(kinetic_energy(psi, grid, order=order))
    V_exp = float(potential_energy(psi, V, grid))
    vr = float(virial_ratio(psi, V, grid, order=order))
    res = HydrogenResult(grid=grid, psi=psi, V=V, energy=T + V_exp, kinetic=T, potential=V_exp, virial_ratio=vr,
                         history=hist)
    if verbose:
        E0 = -0.5 * Z * Z
        print(f"Hydrogenic atom Z={Z} on {N}^3 grid, L = {L}  (h = {grid.h:.4f}, stencil order {order})")
        print(f"Solver        : imag_time   steps = {n_steps}")
        print(f"Energy        : {res.energy:+.6f} Ha     (target: {E0:+.6f})")
        print(f"<T>           : {T:+.6f} Ha     (analytic: {-E0:+.6f})")
        print(f"<V>           : {V_exp:+.6f} Ha     (analytic: {2 * E0:+.6f})")
        print(f"Virial 2T/|V| : {vr:+.6f}        (target:  1.000000)")
    return res
