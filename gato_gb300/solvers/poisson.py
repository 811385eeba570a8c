"""Hartree potential by Hockney doubled-grid FFT convolution (reference: poisson.py:1-92).

A :class:`PoissonPlan` owns the FP64-built spectrum of the softened 1/r
kernel for one (N, h, eps, dtype) and the spectral work buffers; plans are
cached, so the kernel transform happens once (the reference rebuilds it on
every call).
"""
from __future__ import annotations

import ctypes as C
import threading
from collections import OrderedDict

import torch

from .. import _lib
from ..grid import Grid3D, as_field


class PoissonPlan:
    def __init__(self, N: int, h: float, eps: float, dtype=torch.float64, max_fields: int = 6):
        _lib.require_cuda()
        self.N, self.h, self.eps, self.dtype, self.max_fields = N, h, eps, dtype, max_fields
        handle = C.c_void_p()
        _lib.call("gato_poisson_create", _lib.dtype_code(dtype), N, float(h), float(eps), max_fields,
                  C.byref(handle), C.c_void_p(_lib.stream()))
        self.handle = handle

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and _lib._lib is not None:
            _lib._lib.gato_poisson_destroy(h)
            self.handle = None

    def potential(self, rho: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        if out is None:
            out = torch.empty_like(rho)
        _lib.call("gato_hartree_potential", self.handle, C.c_void_p(rho.data_ptr()),
                  C.c_void_p(out.data_ptr()), C.c_void_p(_lib.stream()))
        return out

    def energy(self, rho: torch.Tensor) -> torch.Tensor:
        out = torch.empty((), dtype=torch.float64, device=rho.device)
        _lib.call("gato_hartree_energy", self.handle, C.c_void_p(rho.data_ptr()),
                  C.c_void_p(out.data_ptr()), C.c_void_p(_lib.stream()))
        return out

    def exchange_into(self, psi: torch.Tensor, fields: torch.Tensor, out: torch.Tensor,
                      coef: float = 1.0) -> torch.Tensor:
        """out += coef * sum_j phi_j J[phi_j psi] for fields (n, N, N, N)."""
        _lib.call("gato_exchange_apply", self.handle, C.c_void_p(psi.data_ptr()),
                  C.c_void_p(fields.data_ptr()), fields.shape[0], C.c_void_p(out.data_ptr()),
                  float(coef), C.c_void_p(_lib.stream()))
        return out


# Plans own spectral work buffers, which one stream at a time may use: the
# cache is per thread, so threads driving their own streams never share one.
_TLS = threading.local()


def _plans() -> "OrderedDict[tuple, PoissonPlan]":
    d = getattr(_TLS, "plans", None)
    if d is None:
        d = _TLS.plans = OrderedDict()
    return d


def get_plan(N: int, h: float, eps: float, dtype=torch.float64, max_fields: int = 6) -> PoissonPlan:
    """The calling thread's cached plan for (N, h, eps, dtype), built if absent (3 kept per thread)."""
    _PLANS = _plans()
    key = (N, float(h), float(eps), dtype)
    p = _PLANS.get(key)
    if p is None or p.max_fields < max_fields:
        if p is not None:
            del _PLANS[key]
        p = PoissonPlan(N, h, eps, dtype, max_fields)
        _PLANS[key] = p
        while len(_PLANS) > 3:
            _PLANS.popitem(last=False)
    else:
        _PLANS.move_to_end(key)
    return p


def hartree_potential(rho, grid: Grid3D, epsilon: float | None = None) -> torch.Tensor:
    """J(r) = int rho(r') / |r - r'| dV' with the softened kernel (poisson.py:60-79)."""
    if epsilon is None:
        epsilon = grid.h / 2
    rho = as_field(rho)
    return get_plan(grid.N, grid.h, epsilon, rho.dtype).potential(rho)


def hartree_energy(rho, grid: Grid3D, epsilon: float | None = None) -> torch.Tensor:
    """E_H = 1/2 int rho J[rho] dV (poisson.py:82-92)."""
    if epsilon is None:
        epsilon = grid.h / 2
    rho = as_field(rho)
    return get_plan(grid.N, grid.h, epsilon, rho.dtype).energy(rho)
