"""Alternating SCF + Adam geometry optimisation (reference: geometry_opt.py:28-78).

The reference uses optax.adam; this is Adam as published by Kingma & Ba with
optax's defaults (b1 = 0.9, b2 = 0.999, eps = 1e-8, eps_root = 0), acting on
the (K, 3) host tensor of positions.
"""
from __future__ import annotations

from typing import Callable

import torch

from .geometry import Nuclei, recenter


class Adam:
    def __init__(self, learning_rate: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        self.lr, self.b1, self.b2, self.eps = learning_rate, b1, b2, eps
        self.mu = self.nu = None
        self.count = 0

    def update(self, g: torch.Tensor) -> torch.Tensor:
        g = g.to(torch.float64)
        if self.mu is None:
            self.mu, self.nu = torch.zeros_like(g), torch.zeros_like(g)
        self.count += 1
        self.mu = self.b1 * self.mu + (1 - self.b1) * g
        self.nu = self.b2 * self.nu + (1 - self.b2) * g * g
        mu_hat = self.mu / (1 - self.b1 ** self.count)
        nu_hat = self.nu / (1 - self.b2 ** self.count)
        return -self.lr * mu_hat / (torch.sqrt(nu_hat) + self.eps)


def optimize_geometry_alternating(initial_nuclei: Nuclei, *, solve_at_geometry: Callable,
                                  bo_grad: Callable, geom_steps: int, learning_rate: float = 0.05,
                                  on_step: Callable | None = None):
    """Solve, Adam step on dE/dR, recenter, warm-started re-solve (geometry_opt.py:28-78)."""
    nuclei = recenter(initial_nuclei)
    opt = Adam(learning_rate)
    current = solve_at_geometry(nuclei, None)
    trajectory = [current]
    for step in range(geom_steps):
        grad_R = bo_grad(current)
        upd = opt.update(grad_R)
        nuclei = recenter(Nuclei(current.nuclei.positions + upd, current.nuclei.charges))
        current = solve_at_geometry(nuclei, current)
        if on_step is not None:
            on_step(step, current)
        trajectory.append(current)
    return current, trajectory
