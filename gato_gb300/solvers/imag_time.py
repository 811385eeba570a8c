"""Imaginary-time propagation (reference: solvers/imag_time.py:1-65).

psi <- psi - dt H psi, renormalised, n_steps times: each step is one fused
stencil launch with coefficient dt / (2 h^2) and potential 1 - dt V, a norm
reduction and a rescale, replayed from a CUDA graph inside libgato_cuda.
Stability needs dt < 1 / lambda_max(H) (about h^2 / 6 for the 7-point
Laplacian); the default is dt = h^2 / 10 as in the reference.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from .. import _lib
from ..grid import as_field


@dataclass
class ImagTimeHistory:
    steps: list
    energies: list


def imaginary_time(H, psi0, dt: float | None = None, n_steps: int = 2000, log_every: int = 50):
    """Propagate psi0 in imaginary time toward the ground state of H (imag_time.py:29-65).

    H is a ``Hamiltonian`` (grid, V, boundary, order). Returns (psi, history),
    with the Rayleigh quotient logged after every step i with
    i % log_every == 0 and after the last step.
    """
    grid = H.grid
    if dt is None:
        dt = grid.h ** 2 / 10.0
    psi = as_field(psi0)
    if torch.is_complex(psi):
        raise TypeError("imaginary_time propagates real fields")
    psi = psi.clone()
    V = getattr(H, "V", None)
    V = as_field(V, psi.dtype) if V is not None else None
    steps = [i for i in range(n_steps) if i % log_every == 0 or i == n_steps - 1]
    energies = torch.empty(max(len(steps), 1), dtype=torch.float64, device=psi.device)
    _lib.call("gato_imag_time", _lib.dtype_code(psi), C.c_void_p(psi.data_ptr()),
              C.c_void_p(V.data_ptr() if V is not None else None), grid.N, float(grid.h), int(H.order),
              _lib.boundary_code(H.boundary), float(dt), int(n_steps), int(log_every),
              C.c_void_p(energies.data_ptr()), C.c_void_p(_lib.stream()))
    return psi, ImagTimeHistory(steps, energies[: len(steps)].tolist())
