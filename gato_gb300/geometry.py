"""Nuclear positions, bonds and nuclear repulsion (reference: geometry.py:20-91).

Positions are (K, 3) float64 tensors on the host: a handful of numbers per
molecule, so this module is plain torch arithmetic and differentiable with
torch.autograd, as the reference's is with jax.grad.
"""
from __future__ import annotations

from typing import NamedTuple

import torch


def _t(x):
    return x if isinstance(x, torch.Tensor) else torch.as_tensor(x, dtype=torch.float64)


class Nuclei(NamedTuple):
    """K nuclei: positions (K, 3) in bohr, charges (K,)."""

    positions: torch.Tensor
    charges: torch.Tensor

    @property
    def n(self) -> int:
        return int(self.charges.shape[0])


def diatomic_along_z(R: float, Z1: float, Z2: float | None = None) -> Nuclei:
    if Z2 is None:
        Z2 = Z1
    return Nuclei(torch.tensor([[0.0, 0.0, -R / 2], [0.0, 0.0, R / 2]], dtype=torch.float64),
                  torch.tensor([Z1, Z2], dtype=torch.float64))


def bond_length(nuclei: Nuclei, i: int, j: int) -> torch.Tensor:
    return torch.linalg.norm(_t(nuclei.positions)[i] - _t(nuclei.positions)[j])


def bond_angle(nuclei: Nuclei, i: int, j: int, k: int) -> torch.Tensor:
    p = _t(nuclei.positions)
    a, b = p[i] - p[j], p[k] - p[j]
    c = torch.dot(a, b) / (torch.linalg.norm(a) * torch.linalg.norm(b))
    return torch.arccos(torch.clamp(c, -1.0, 1.0))


def nuclear_repulsion(nuclei: Nuclei) -> torch.Tensor:
    """E_nn = sum_{i<j} Z_i Z_j / |R_i - R_j| (geometry.py:61-75)."""
    p, q = _t(nuclei.positions), _t(nuclei.charges)
    K = q.shape[0]
    if K < 2:
        return torch.zeros((), dtype=p.dtype)
    i, j = torch.triu_indices(K, K, offset=1)
    r = torch.linalg.norm(p[i] - p[j], dim=-1)
    return torch.sum(q[i] * q[j] / r)


def center_of_mass(nuclei: Nuclei) -> torch.Tensor:
    p, q = _t(nuclei.positions), _t(nuclei.charges)
    return (q[:, None] * p).sum(dim=0) / q.sum()


def recenter(nuclei: Nuclei) -> Nuclei:
    return Nuclei(_t(nuclei.positions) - center_of_mass(nuclei), _t(nuclei.charges))
