"""Finite-difference Laplacian and kinetic operator (reference: operators.py:40-130).

``order=2`` is the 7-point stencil, ``order=4`` the 13-point one; Dirichlet
means zero outside the grid, periodic wraps. Both run in one libgato_cuda
kernel (TMA-staged plane marching on the Dirichlet path). Complex fields are
applied part by part (the stencil is real).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .grid import as_field


def _check(order: int, boundary: str) -> int:
    if order not in (2, 4):
        raise ValueError(f"Unknown order {order!r}; expected 2 or 4.")
    return _lib.boundary_code(boundary)


def stencil(psi, h: float, boundary: str, order: int, coef: float, V=None, out=None,
            dot: bool = False):
    """out = coef * L(psi) + V * psi for psi of shape (nx, ny, nz) or (nb, nx, ny, nz).

    With dot=True also returns the per-field <psi, out> dV (the Hamiltonian
    expectation) as float64 CUDA tensor(s).
    """
    bcode = _check(order, boundary)
    psi = as_field(psi)
    if torch.is_complex(psi):
        if V is not None and torch.is_complex(V):
            raise TypeError("complex potentials are not supported")
        re = stencil(psi.real, h, boundary, order, coef, V)
        im = stencil(psi.imag, h, boundary, order, coef, V)
        return torch.complex(re, im)
    if psi.dim() == 3:
        nb, (nx, ny, nz) = 1, psi.shape
    elif psi.dim() == 4:
        nb, nx, ny, nz = psi.shape
    else:
        raise ValueError(f"expected a 3-D field or a 4-D block of fields, got shape {tuple(psi.shape)}")
    if V is not None:
        V = as_field(V, psi.dtype)
        if tuple(V.shape) != (nx, ny, nz):
            raise ValueError("potential shape does not match the field")
    if out is None:
        out = torch.empty_like(psi)
    dots = torch.empty(nb, dtype=torch.float64, device=psi.device) if dot else None
    _lib.call("gato_stencil_apply", _lib.dtype_code(psi), C.c_void_p(psi.data_ptr()),
              C.c_void_p(V.data_ptr() if V is not None else None), C.c_void_p(out.data_ptr()),
              nb, nx, ny, nz, coef, bcode, order,
              C.c_void_p(dots.data_ptr() if dots is not None else None), h ** 3,
              C.c_void_p(_lib.stream()))
    if dot:
        return out, (dots[0] if psi.dim() == 3 else dots)
    return out


def laplacian(psi, h: float, boundary: str = "dirichlet", order: int = 2) -> torch.Tensor:
    """Central-difference 3-D Laplacian (operators.py:40-119)."""
    _check(order, boundary)
    return stencil(psi, h, boundary, order, 1.0 / (h * h))


def kinetic(psi, h: float, boundary: str = "dirichlet", order: int = 2) -> torch.Tensor:
    """T psi = -1/2 Laplacian psi (operators.py:122-130)."""
    _check(order, boundary)
    return stencil(psi, h, boundary, order, -0.5 / (h * h))
