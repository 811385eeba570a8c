"""Geometry optimisation loop shared by the diatomic drivers (lih.py:218-266, hcl.py:234-283,
h2.py:157-214): alternating warm-started SCF and Adam on the Hellmann-Feynman gradient, with a
(step, energy, bond length) trajectory."""
from __future__ import annotations

from ..geometry import bond_length
from ..geometry_opt import optimize_geometry_alternating


def optimize_diatomic(initial_nuclei, solve_at, bo_grad, *, geom_steps: int, learning_rate: float,
                      label: str, verbose: bool):
    trajectory: list[tuple[int, float, float]] = []

    def on_step(step, p):
        R = float(bond_length(p.nuclei, 0, 1))
        trajectory.append((step, p.energy, R))
        if verbose:
            print(f"  geom step {step:3d}  E = {p.energy:+.6f}  {label} = {R:.4f} a0  SCF iters = {p.n_iters}")

    final, _ = optimize_geometry_alternating(initial_nuclei, solve_at_geometry=solve_at, bo_grad=bo_grad,
                                             geom_steps=geom_steps, learning_rate=learning_rate,
                                             on_step=on_step)
    return final, trajectory
