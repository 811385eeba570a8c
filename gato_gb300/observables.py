"""Observables: kinetic / potential energy, virial ratio, radial density (reference: observables.py:1-59).

Every observable divides by <psi|psi>, so psi need not be normalised. The
kinetic term is the stencil kernel's fused <psi|T psi> reduction, the
potential term a weighted dot, the radial density a device histogram with
numpy.histogram's binning.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .grid import Grid3D, as_field, norm_sq
from .operators import stencil


def _real_norm(psi, grid: Grid3D) -> torch.Tensor:
    return norm_sq(psi, grid).real


def kinetic_energy(psi, grid: Grid3D, boundary: str = "dirichlet", order: int = 2) -> torch.Tensor:
    """<T> = <psi|(-1/2 Laplacian)|psi> / <psi|psi> (observables.py:16-21)."""
    psi = as_field(psi)
    if torch.is_complex(psi):
        return (kinetic_energy(psi.real.contiguous(), grid, boundary, order) * _real_norm(psi.real, grid)
                + kinetic_energy(psi.imag.contiguous(), grid, boundary, order) * _real_norm(psi.imag, grid)
                ) / _real_norm(psi, grid)
    _, e = stencil(psi, grid.h, boundary, order, -0.5 / grid.h ** 2, dot=True)
    return e / _real_norm(psi, grid)


def potential_energy(psi, V, grid: Grid3D) -> torch.Tensor:
    """<V> = <psi|V|psi> / <psi|psi> for a multiplicative V (observables.py:24-28)."""
    psi = as_field(psi)
    parts = (psi.real.contiguous(), psi.imag.contiguous()) if torch.is_complex(psi) else (psi,)
    V = as_field(V, parts[0].dtype)
    out = torch.zeros(1, dtype=torch.float64, device=psi.device)
    acc = torch.zeros((), dtype=torch.float64, device=psi.device)
    for p in parts:
        _lib.call("gato_dot_weighted", _lib.dtype_code(p), C.c_void_p(p.data_ptr()), C.c_void_p(V.data_ptr()),
                  C.c_void_p(p.data_ptr()), p.numel(), float(grid.dV), C.c_void_p(out.data_ptr()),
                  C.c_void_p(_lib.stream()))
        acc = acc + out[0]
    return acc / _real_norm(psi, grid)


def virial_ratio(psi, V, grid: Grid3D, boundary: str = "dirichlet", order: int = 2) -> torch.Tensor:
    """2<T> / |<V>| (observables.py:31-44): +1 for a Coulomb eigenstate, 2 for the oscillator."""
    return 2 * kinetic_energy(psi, grid, boundary, order) / torch.abs(potential_energy(psi, V, grid))


def radial_density(psi, grid: Grid3D, n_bins: int = 100, r_max: float | None = None):
    """(r_centers, P) with int P dr = <psi|psi> over [0, r_max] (observables.py:47-59)."""
    psi = as_field(psi)
    re, im = (psi.real.contiguous(), psi.imag.contiguous()) if torch.is_complex(psi) else (psi, None)
    if r_max is None:
        r_max = float(grid.L / 2)
    bins = np.linspace(0.0, r_max, n_bins + 1)
    hist = torch.empty(n_bins, dtype=torch.float64, device=psi.device)
    _lib.call("gato_radial_density", _lib.dtype_code(re), C.c_void_p(re.data_ptr()),
              C.c_void_p(im.data_ptr() if im is not None else None), grid.N, float(grid.L),
              _lib.dbl_array(bins), n_bins, C.c_void_p(hist.data_ptr()), C.c_void_p(_lib.stream()))
    centers = 0.5 * (bins[1:] + bins[:-1])
    widths = bins[1:] - bins[:-1]
    return (torch.tensor(centers, dtype=torch.float64, device=psi.device),
            hist / torch.tensor(widths, dtype=torch.float64, device=psi.device))
