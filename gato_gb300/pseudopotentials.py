"""HGH norm-conserving pseudopotentials (reference: pseudopotentials.py:81-405).

The parameter tables are the published Hartwigsen-Goedecker-Hutter (1998)
LDA values the reference tabulates; they are physical data and must match
for parity. The local part is evaluated on the grid by one kernel; the
non-local part is an :class:`HGHNonlocal` object holding its projectors on
per-atom boxes on the device, callable as ``psi -> V_nl psi`` like the
reference's ``V_nl_apply`` closure.
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from collections import OrderedDict
from dataclasses import dataclass

import torch

from . import _lib
from .geometry import Nuclei, _t
from .grid import Grid3D, as_field

# Gaussian box radius in units of the widest r_l of an atom: the projector
# tail beyond it is below 1e-20 of its peak.
CUT_SIGMAS = 10.0


@dataclass(frozen=True)
class HGHProjector:
    ell: int
    r: float
    h: tuple

    @property
    def n(self) -> int:
        return len(self.h)


@dataclass(frozen=True)
class HGHParams:
    symbol: str
    Z_ion: float
    r_loc: float
    c: tuple
    projectors: tuple = ()


HYDROGEN_HGH = HGHParams("H", 1.0, 0.2, (-4.0663326, 0.6778322, 0.0, 0.0), ())
OXYGEN_HGH = HGHParams("O", 6.0, 0.24762086, (-16.5803180, 2.39570952, 0.0, 0.0),
                       (HGHProjector(0, 0.22178614, ((18.26691718,),)),))
LITHIUM_HGH = HGHParams("Li", 1.0, 0.78755305, (-1.89261247, 0.28605968, 0.0, 0.0),
                        (HGHProjector(0, 0.66637518, ((1.85881111,),)),
                         HGHProjector(1, 1.07930561, ((-0.00589504,),))))
CHLORINE_HGH = HGHParams("Cl", 7.0, 0.41, (-6.86475431, 0.0, 0.0, 0.0),
                         (HGHProjector(0, 0.33820832, ((9.06223968, -1.96193036),
                                                       (-1.96193036, 5.06568240))),
                          HGHProjector(1, 0.37613709, ((4.46587640,),))))
HGH_TABLE = {"H": HYDROGEN_HGH, "Li": LITHIUM_HGH, "O": OXYGEN_HGH, "Cl": CHLORINE_HGH}


def lookup(symbol: str) -> HGHParams:
    """pseudopotentials.py:188-194: KeyError for an unknown element."""
    if symbol not in HGH_TABLE:
        raise KeyError(f"No HGH parameters for {symbol!r}. Add them to gato_gb300.pseudopotentials "
                       f"from Hartwigsen-Goedecker-Hutter 1998 table I.")
    return HGH_TABLE[symbol]


def total_valence_charge(elements) -> float:
    return float(sum(p.Z_ion for p in elements))


def _check_elements(nuclei: Nuclei, elements) -> None:
    if len(elements) != nuclei.n:
        raise ValueError(f"HGH parameter list length {len(elements)} != number of nuclei {nuclei.n}")


def _pos_list(nuclei: Nuclei):
    return [float(v) for v in _t(nuclei.positions).detach().reshape(-1)]


def hgh_local_potential(nuclei: Nuclei, elements, grid: Grid3D, dtype=torch.float64) -> torch.Tensor:
    """Sum of HGH local parts (pseudopotentials.py:230-253), evaluated in FP64."""
    _check_elements(nuclei, elements)
    dev = _lib.require_cuda()
    V = torch.empty(grid.shape, dtype=dtype, device=dev)
    _lib.call("gato_hgh_local", _lib.dtype_code(dtype), C.c_void_p(V.data_ptr()), grid.N,
              float(grid.L), nuclei.n, _lib.dbl_array(_pos_list(nuclei)),
              _lib.dbl_array([p.Z_ion for p in elements]), _lib.dbl_array([p.r_loc for p in elements]),
              _lib.dbl_array([c for p in elements for c in p.c]), C.c_void_p(_lib.stream()))
    return V


def hgh_local_grad(nuclei: Nuclei, elements, grid: Grid3D, rho) -> torch.Tensor:
    """d/dR of int rho V_loc(R) dV, shape (K, 3) (float64, host)."""
    _check_elements(nuclei, elements)
    rho = as_field(rho)
    g = (C.c_double * (3 * nuclei.n))()
    _lib.call("gato_hgh_local_grad", _lib.dtype_code(rho), C.c_void_p(rho.data_ptr()), grid.N,
              float(grid.L), nuclei.n, _lib.dbl_array(_pos_list(nuclei)),
              _lib.dbl_array([p.Z_ion for p in elements]), _lib.dbl_array([p.r_loc for p in elements]),
              _lib.dbl_array([c for p in elements for c in p.c]), g, C.c_void_p(_lib.stream()))
    return torch.tensor(list(g), dtype=torch.float64).reshape(nuclei.n, 3)


class HGHNonlocal:
    """Device-resident separable non-local operator of one geometry.

    ``nl(psi)`` returns V_nl psi (pseudopotentials.py:360-383) for one field
    or a block of fields stacked on the first axis.
    """

    def __init__(self, nuclei: Nuclei, elements, grid: Grid3D, dtype=torch.float64):
        _check_elements(nuclei, elements)
        _lib.require_cuda()
        self.grid, self.dtype, self.nuclei, self.elements = grid, dtype, nuclei, tuple(elements)
        nch, ell, r, n, h = [], [], [], [], []
        for p in elements:
            nch.append(len(p.projectors))
            for pr in p.projectors:
                ell.append(pr.ell)
                r.append(pr.r)
                n.append(pr.n)
                m = [0.0] * 9
                for i in range(pr.n):
                    for j in range(pr.n):
                        m[3 * i + j] = float(pr.h[i][j])
                h.extend(m)
        self.n_channels = len(ell)
        handle = C.c_void_p()
        _lib.call("gato_nonlocal_create", _lib.dtype_code(dtype), grid.N, float(grid.L), nuclei.n,
                  _lib.dbl_array(_pos_list(nuclei)), _lib.int_array(nch), _lib.int_array(ell),
                  _lib.dbl_array(r), _lib.int_array(n), _lib.dbl_array(h), CUT_SIGMAS, C.byref(handle))
        self.handle = handle

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and _lib._lib is not None:
            _lib._lib.gato_nonlocal_destroy(h)
            self.handle = None

    def add_to(self, psi: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        nb = 1 if psi.dim() == 3 else psi.shape[0]
        _lib.call("gato_nonlocal_apply", self.handle, C.c_void_p(psi.data_ptr()),
                  C.c_void_p(out.data_ptr()), nb, C.c_void_p(_lib.stream()))
        return out

    def __call__(self, psi) -> torch.Tensor:
        psi = as_field(psi, self.dtype)
        return self.add_to(psi, torch.zeros_like(psi))

    def energy(self, fields: torch.Tensor) -> torch.Tensor:
        """2 sum_b <psi_b|V_nl|psi_b> for a (n, N, N, N) block."""
        out = torch.empty((), dtype=torch.float64, device=fields.device)
        _lib.call("gato_nonlocal_energy", self.handle, C.c_void_p(fields.data_ptr()), fields.shape[0],
                  C.c_void_p(out.data_ptr()), C.c_void_p(_lib.stream()))
        return out

    def grad(self, fields: torch.Tensor) -> torch.Tensor:
        """d/dR of 2 sum_b <psi_b|V_nl(R)|psi_b>, shape (K, 3), host float64."""
        K = self.nuclei.n
        g = (C.c_double * (3 * K))()
        _lib.call("gato_nonlocal_grad", self.handle, C.c_void_p(fields.data_ptr()), fields.shape[0], g,
                  C.c_void_p(_lib.stream()))
        return torch.tensor(list(g), dtype=torch.float64).reshape(K, 3)


# Per-thread, like the Poisson plans: an operator's projection scratch serves one stream at a time.
_NL_TLS = threading.local()


def nonlocal_for(nuclei: Nuclei, elements, grid: Grid3D, dtype=torch.float64) -> HGHNonlocal:
    key = (tuple(_pos_list(nuclei)), tuple(p.symbol for p in elements), tuple(id(p) for p in elements),
           grid.N, float(grid.L), dtype)
    _NL_CACHE = getattr(_NL_TLS, "cache", None)
    if _NL_CACHE is None:
        _NL_CACHE = _NL_TLS.cache = OrderedDict()
    nl = _NL_CACHE.get(key)
    if nl is None:
        nl = HGHNonlocal(nuclei, elements, grid, dtype)
        _NL_CACHE[key] = nl
        while len(_NL_CACHE) > 4:
            _NL_CACHE.popitem(last=False)
    else:
        _NL_CACHE.move_to_end(key)
    return nl


def hgh_nonlocal_apply(psi, nuclei: Nuclei, elements, grid: Grid3D) -> torch.Tensor:
    """(V_nl psi) (pseudopotentials.py:360-383)."""
    psi = as_field(psi)
    return nonlocal_for(nuclei, elements, grid, psi.dtype)(psi)


def hgh_apply(psi, nuclei: Nuclei, elements, grid: Grid3D, V_local=None) -> torch.Tensor:
    """V_loc psi + V_nl psi (pseudopotentials.py:390-405)."""
    psi = as_field(psi)
    if V_local is None:
        V_local = hgh_local_potential(nuclei, elements, grid, psi.dtype)
    return as_field(V_local, psi.dtype) * psi + hgh_nonlocal_apply(psi, nuclei, elements, grid)


def _projector_radial(r, ell: int, i_idx: int, r_ell: float):
    """Radial HGH projector p_li(r) (pseudopotentials.py:265-277), for 1-D checks."""
    n = ell + (4 * i_idx - 1) / 2.0
    norm = math.sqrt(2.0) / (r_ell ** n * math.sqrt(math.gamma(n)))
    r = torch.as_tensor(r, dtype=torch.float64)
    return norm * (r ** (ell + 2 * (i_idx - 1))) * torch.exp(-(r * r) / (2.0 * r_ell * r_ell))
