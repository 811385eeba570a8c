"""Cell-centred Cartesian grid and FP64 reductions (reference: grid.py:1-73).

Fields are CUDA tensors of shape (N, N, N), C-order with z fastest. The
reductions run in libgato_cuda (FP64 accumulation; float-float for float32
fields) and return 0-d float64 CUDA tensors, so nothing synchronises until
the caller converts them with ``float()``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib


@dataclass(frozen=True)
class Grid3D:
    """Uniform cell-centred grid on [-L/2, L/2]^3, x_i = -L/2 + (i + 1/2) h."""

    N: int
    L: float

    @property
    def h(self) -> float:
        return self.L / self.N

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.N, self.N, self.N)

    @property
    def dV(self) -> float:
        return self.h ** 3

    def axis(self, dtype=torch.float64) -> torch.Tensor:
        dev = _lib.require_cuda()
        a = -self.L / 2 + (torch.arange(self.N, dtype=torch.float64) + 0.5) * self.h   # host, then one copy
        return a.to(dtype).to(dev)

    def coords(self, dtype=torch.float64):
        a = self.axis(dtype)
        return torch.meshgrid(a, a, a, indexing="ij")

    def radial(self, softening: float = 0.0) -> torch.Tensor:
        X, Y, Z = self.coords()
        return torch.sqrt(X * X + Y * Y + Z * Z + softening * softening)


_CONVERTIBLE = (torch.float32, torch.float64)


def as_field(x, dtype=None) -> torch.Tensor:
    """A contiguous CUDA tensor view/copy of x (numpy, CPU or CUDA tensor).

    Host data is converted and made contiguous on the host and copied once; a contiguous device field
    changes between FP32 and FP64 through the library's conversion kernel."""
    dev = _lib.require_cuda()
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(x)
    if x.device != dev:
        if dtype is not None and x.dtype != dtype:
            x = x.to(dtype)
        return x.contiguous().to(dev)
    if dtype is not None and x.dtype != dtype:
        if x.is_contiguous() and x.numel() > 0 and x.dtype in _CONVERTIBLE and dtype in _CONVERTIBLE:
            out = torch.empty(x.shape, dtype=dtype, device=dev)
            _lib.call("gato_convert", _lib.dtype_code(x), C.c_void_p(x.data_ptr()), _lib.dtype_code(out),
                      C.c_void_p(out.data_ptr()), x.numel(), C.c_void_p(_lib.stream()))
            return out
        x = x.to(dtype)
    return x.contiguous()


def _dot(a: torch.Tensor, b, scale: float) -> torch.Tensor:
    out = torch.empty((), dtype=torch.float64, device=a.device)
    _lib.call("gato_dot", _lib.dtype_code(a), C.c_void_p(a.data_ptr()),
              C.c_void_p(b.data_ptr() if b is not None else None), a.numel(), scale,
              C.c_void_p(out.data_ptr()), C.c_void_p(_lib.stream()))
    return out


def _real_parts(x):
    if torch.is_complex(x):
        return x.real.contiguous(), x.imag.contiguous()
    return x, None


def integrate(psi, grid: Grid3D) -> torch.Tensor:
    """Midpoint-rule integral sum(psi) dV (grid.py:57-59)."""
    psi = as_field(psi)
    re, im = _real_parts(psi)
    r = _dot(re, None, grid.dV)
    if im is None:
        return r
    return torch.complex(r, _dot(im, None, grid.dV))


def inner_product(phi, psi, grid: Grid3D) -> torch.Tensor:
    """<phi|psi> = sum(conj(phi) psi) dV (grid.py:62-64)."""
    phi, psi = as_field(phi), as_field(psi)
    if not torch.is_complex(phi) and not torch.is_complex(psi):
        return _dot(phi, psi, grid.dV)
    pr, pi = _real_parts(phi)
    qr, qi = _real_parts(psi)
    re = _dot(pr, qr, grid.dV)
    im = torch.zeros((), dtype=torch.float64, device=re.device)
    if pi is not None and qi is not None:
        re = re + _dot(pi, qi, grid.dV)
    if qi is not None:
        im = im + _dot(pr, qi, grid.dV)
    if pi is not None:
        im = im - _dot(pi, qr, grid.dV)
    return torch.complex(re, im)


def norm_sq(psi, grid: Grid3D) -> torch.Tensor:
    """sum |psi|^2 dV (grid.py:67-69)."""
    psi = as_field(psi)
    re, im = _real_parts(psi)
    r = _dot(re, re, grid.dV)
    if im is not None:
        r = r + _dot(im, im, grid.dV)
    return r


def normalize(psi, grid: Grid3D) -> torch.Tensor:
    """psi / sqrt(norm_sq(psi)) (grid.py:72-73)."""
    psi = as_field(psi)
    if torch.is_complex(psi):
        n = norm_sq(psi, grid)
        return psi / torch.sqrt(n)
    out = psi.clone()
    n = _dot(psi, psi, grid.dV)
    _lib.call("gato_normalize", _lib.dtype_code(out), C.c_void_p(out.data_ptr()), out.numel(),
              C.c_void_p(n.data_ptr()), C.c_void_p(_lib.stream()))
    return out
