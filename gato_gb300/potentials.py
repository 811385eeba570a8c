"""External potentials sampled on the grid (reference: potentials.py:16-76)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .geometry import Nuclei, _t
from .grid import Grid3D


def _softened(grid: Grid3D, pos, Z, eps: float, dtype) -> torch.Tensor:
    dev = _lib.require_cuda()
    V = torch.empty(grid.shape, dtype=dtype, device=dev)
    pos = [float(v) for v in torch.as_tensor(pos, dtype=torch.float64).reshape(-1)]
    Z = [float(v) for v in torch.as_tensor(Z, dtype=torch.float64).reshape(-1)]
    _lib.call("gato_softened_coulomb", _lib.dtype_code(dtype), C.c_void_p(V.data_ptr()), grid.N,
              float(grid.L), len(Z), _lib.dbl_array(pos), _lib.dbl_array(Z), float(eps),
              C.c_void_p(_lib.stream()))
    return V


def softened_coulomb(grid: Grid3D, Z: float = 1.0, epsilon: float | None = None,
                     center=(0.0, 0.0, 0.0), dtype=torch.float64) -> torch.Tensor:
    """V = -Z / sqrt(|r - r0|^2 + eps^2), eps defaulting to h/2 (potentials.py:16-36)."""
    if epsilon is None:
        epsilon = grid.h / 2
    return _softened(grid, [center], [Z], epsilon, dtype)


def multi_center_softened_coulomb(nuclei: Nuclei, grid: Grid3D, epsilon: float | None = None,
                                  dtype=torch.float64) -> torch.Tensor:
    """V = -sum_k Z_k / sqrt(|r - R_k|^2 + eps^2) (potentials.py:39-61)."""
    if epsilon is None:
        epsilon = grid.h / 2
    return _softened(grid, _t(nuclei.positions).detach(), _t(nuclei.charges).detach(), epsilon, dtype)


def multi_center_softened_coulomb_grad(nuclei: Nuclei, grid: Grid3D, rho, epsilon: float | None = None
                                       ) -> torch.Tensor:
    """d/dR of int rho V_ext dV for the multi-centre softened Coulomb V_ext, (K, 3) float64 host.

    The force term the reference obtains with jax.grad through
    multi_center_softened_coulomb (physics/h2.py:109-135).
    """
    from .grid import as_field
    if epsilon is None:
        epsilon = grid.h / 2
    rho = as_field(rho)
    pos = [float(v) for v in _t(nuclei.positions).detach().to(torch.float64).reshape(-1)]
    Z = [float(v) for v in _t(nuclei.charges).detach().to(torch.float64).reshape(-1)]
    g = (C.c_double * (3 * len(Z)))()
    _lib.call("gato_softened_coulomb_grad", _lib.dtype_code(rho), C.c_void_p(rho.data_ptr()), grid.N,
              float(grid.L), len(Z), _lib.dbl_array(pos), _lib.dbl_array(Z), float(epsilon), g,
              C.c_void_p(_lib.stream()))
    return torch.tensor(list(g), dtype=torch.float64).reshape(len(Z), 3)


def harmonic_oscillator(grid: Grid3D, omega: float = 1.0) -> torch.Tensor:
    """1/2 omega^2 r^2 (potentials.py:64-69); a test fixture."""
    X, Y, Z = grid.coords()
    return 0.5 * omega * omega * (X * X + Y * Y + Z * Z)


def constant(grid: Grid3D, v0: float = 0.0) -> torch.Tensor:
    """Uniform v0 (potentials.py:72-76); a test fixture."""
    return torch.full(grid.shape, float(v0), dtype=torch.float64, device=_lib.require_cuda())
