"""Single-particle Hamiltonian H = T + V (reference: hamiltonian.py:18-35)."""
from __future__ import annotations

from dataclasses import dataclass

import torch

from .grid import Grid3D, as_field, norm_sq
from .operators import stencil


@dataclass(frozen=True)
class Hamiltonian:
    grid: Grid3D
    V: torch.Tensor
    boundary: str = "dirichlet"
    order: int = 2

    def apply(self, psi) -> torch.Tensor:
        """H psi = (-1/2 Laplacian + V) psi in one fused kernel."""
        return stencil(psi, self.grid.h, self.boundary, self.order, -0.5 / self.grid.h ** 2,
                       V=self.V)

    def expectation(self, psi) -> torch.Tensor:
        """<psi|H|psi>, reduced inside the stencil kernel."""
        _, e = stencil(psi, self.grid.h, self.boundary, self.order, -0.5 / self.grid.h ** 2,
                       V=self.V, dot=True)
        return e

    def rayleigh(self, psi) -> torch.Tensor:
        psi = as_field(psi)
        return self.expectation(psi) / norm_sq(psi, self.grid)

    def _gato_operator(self, dtype):
        from .scf import Operator
        op = Operator(self.grid, dtype, self.order, self.boundary)
        op.set_potential(as_field(self.V, dtype))
        return op
