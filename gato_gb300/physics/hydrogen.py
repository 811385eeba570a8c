"""One-electron atom in imaginary time (reference counterpart: physics/hydrogen.py).

The softened Coulomb well of charge Z at the box centre is relaxed to its
ground state by ``imaginary_time`` (a replayed fused Euler step on the
device); the result carries the normalised state and its kinetic and
potential expectation values. The exact nonrelativistic ground-state energy
of the unsoftened well is -Z^2 / 2 Ha, and a Coulomb eigenstate has
2<T> / |<V>| = 1.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from ..ansatz import init_grid_ansatz
from ..grid import Grid3D, normalize
from ..hamiltonian import Hamiltonian
from ..observables import kinetic_energy, potential_energy
from ..potentials import softened_coulomb
from ..solvers.imag_time import imaginary_time


@dataclass
class HydrogenResult:
    """Field names as in the reference's result record (hydrogen.py:27-36)."""

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
    """Ground state of charge Z by imaginary time from a hydrogenic start (seeded)."""
    grid = Grid3D(N=N, L=L)
    well = softened_coulomb(grid, Z=Z, epsilon=epsilon)
    start = init_grid_ansatz(grid, seed, init="hydrogenic", Z=Z)
    state, log = imaginary_time(Hamiltonian(grid=grid, V=well, order=order), start, n_steps=n_steps,
                                log_every=max(1, n_steps // 20))
    state = normalize(state, grid)
    t = float(kinetic_energy(state, grid, order=order))
    v = float(potential_energy(state, well, grid))
    out = HydrogenResult(grid=grid, psi=state, V=well, energy=t + v, kinetic=t, potential=v,
                         virial_ratio=2.0 * t / abs(v), history=list(zip(log.steps, log.energies)))
    if verbose:
        print(f"hydrogenic Z={Z:g} N={N} L={L:g} order={order} steps={n_steps}: E={out.energy:.6f} Ha "
              f"(exact {-0.5 * Z * Z:.6f}), T={t:.6f}, V={v:.6f}, 2T/|V|={out.virial_ratio:.5f}")
    return out
