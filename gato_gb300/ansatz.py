"""Starting fields on the grid (reference: ansatz/grid.py:16-48).

``key`` is an integer seed for a torch generator (the reference takes a JAX
PRNG key); it only matters for init="random" and for noise > 0, whose draws
therefore differ from the reference's. "hydrogenic" and "gaussian" without
noise are the same fields.
"""
from __future__ import annotations

import torch

from . import _lib
from .grid import Grid3D


def init_grid_ansatz(grid: Grid3D, key: int = 0, init: str = "hydrogenic", Z: float = 1.0,
                     noise: float = 0.0) -> torch.Tensor:
    """exp(-Z sqrt(r^2 + (h/2)^2)) ("hydrogenic"), exp(-r^2/2) ("gaussian") or unit normals ("random")."""
    dev = _lib.require_cuda()
    gen = torch.Generator(device=dev).manual_seed(int(key))
    if init == "hydrogenic":
        psi = torch.exp(-Z * grid.radial(softening=grid.h / 2))
    elif init == "gaussian":
        r = grid.radial()
        psi = torch.exp(-r * r / 2)
    elif init == "random":
        return torch.randn(grid.shape, generator=gen, dtype=torch.float64, device=dev)
    else:
        raise ValueError(f"Unknown init {init!r}")
    if noise > 0:
        psi = psi + noise * torch.randn(grid.shape, generator=gen, dtype=torch.float64, device=dev)
    return psi.contiguous()
