"""Restricted Hartree-Fock SCF on the grid (reference: scf.py:1-444).

Orbitals are stored field-major, (n, N, N, N); the reference's (N, N, N, n)
arrays are the ``permute(1, 2, 3, 0)`` view of that storage, and both forms
are accepted. ``precision="mixed"`` runs the Fock operator (stencils, FFTs, exchange) and
the Lanczos vectors in FP32 with FP64 / float-float reductions, FP64 Lanczos
coefficients and an FP64 tridiagonal eigensolve, and keeps the SCF density,
V_H and the energy in FP64; ``"fp64"`` is the plain path.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Callable

import torch

from . import _lib
from .grid import Grid3D, as_field, inner_product
from .hamiltonian import Hamiltonian
from .operators import kinetic
from .pseudopotentials import HGHNonlocal, nonlocal_for
from .solvers.lanczos import default_krylov_dim, lanczos
from .solvers.poisson import get_plan, hartree_potential

PRECISIONS = {"fp64": torch.float64, "mixed": torch.float32}


def precision_dtype(precision: str) -> torch.dtype:
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be 'fp64' or 'mixed', got {precision!r}")
    return PRECISIONS[precision]


def to_fields(orbitals, dtype=None) -> torch.Tensor:
    """(N, N, N, n) orbitals -> contiguous (n, N, N, N) block (no copy if already so)."""
    if not isinstance(orbitals, torch.Tensor):
        orbitals = torch.as_tensor(orbitals)
    f = orbitals.permute(3, 0, 1, 2)
    dev = _lib.require_cuda()
    if f.is_contiguous() and f.device == dev and (dtype is None or f.dtype == dtype):
        return f
    return as_field(f, dtype)


def from_fields(fields: torch.Tensor) -> torch.Tensor:
    return fields.permute(1, 2, 3, 0)


def pair_fields(n: int) -> int:
    """Complex fields for the energy pass: n(n+1)/2 pairs plus the density."""
    return (n * (n + 1) // 2 + 2) // 2


class Operator:
    """Handle on a libgato_cuda operator: F = -1/2 L + V [+ V_nl] [- K]."""

    def __init__(self, grid: Grid3D, dtype, order: int = 4, boundary: str = "dirichlet"):
        _lib.require_cuda()
        self.grid, self.dtype = grid, dtype
        h = C.c_void_p()
        _lib.call("gato_op_create", _lib.dtype_code(dtype), grid.N, float(grid.h), order,
                  _lib.boundary_code(boundary), C.byref(h))
        self.handle = h
        self._keep = {}

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and _lib._lib is not None:
            _lib._lib.gato_op_destroy(h)
            self.handle = None

    block_epilogue = 0   # 0 auto, 1 J fields + pair pass, 2 fused accumulation (see gato_op_tune)

    def tune(self, block_epilogue: int):
        _lib.call("gato_op_tune", self.handle, int(block_epilogue))
        self.block_epilogue = int(block_epilogue)

    def overlap(self, on: bool):
        """Run the stencil and non-local part beside the exchange transforms (True, the default) or
        in order on the caller's stream (False); results are the same either way."""
        _lib.call("gato_op_overlap", self.handle, int(bool(on)))

    def set_potential(self, V: torch.Tensor | None):
        self._keep["V"] = V
        _lib.call("gato_op_set_potential", self.handle, C.c_void_p(V.data_ptr() if V is not None else None))

    def set_nonlocal(self, nl: HGHNonlocal | None):
        self._keep["nl"] = nl
        _lib.call("gato_op_set_nonlocal", self.handle, nl.handle if nl is not None else None)

    def set_exchange(self, plan, fields: torch.Tensor | None):
        self._keep["plan"], self._keep["orb"] = plan, fields
        n = 0 if fields is None else fields.shape[0]
        _lib.call("gato_op_set_exchange", self.handle, plan.handle if plan is not None else None,
                  C.c_void_p(fields.data_ptr() if fields is not None else None), n)

    def apply(self, psi: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        if out is None:
            out = torch.empty_like(psi)
        _lib.call("gato_op_apply", self.handle, C.c_void_p(psi.data_ptr()), C.c_void_p(out.data_ptr()),
                  C.c_void_p(_lib.stream()))
        return out

    def apply_block(self, out: torch.Tensor | None = None) -> torch.Tensor:
        """F phi_i for the operator's own orbitals, with n(n+1)/2 pair solves."""
        orb = self._keep["orb"]
        if out is None:
            out = torch.empty_like(orb)
        _lib.call("gato_op_apply_block", self.handle, C.c_void_p(out.data_ptr()), C.c_void_p(_lib.stream()))
        return out

    def block_graph(self, out: torch.Tensor) -> torch.cuda.CUDAGraph:
        """``apply_block(out)`` captured once as a CUDA graph; ``replay()`` re-runs its launches.

        The graph holds the addresses of the orbitals, potential, projectors, plan
        buffers and ``out``: their values may change between replays, their
        storage may not, and a later ``set_*``/``tune`` call (or a plan or stencil
        tuning change) needs a new graph. A warm-up run first lets the operator
        allocate its pair-potential buffer, so nothing allocates inside the graph;
        the block apply uses no per-stream scratch. Replays on one stream at a
        time: the plan's spectral buffers and the projector object are shared."""
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.apply_block(out)
        torch.cuda.current_stream().wait_stream(side)
        with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
            self.apply_block(out)
        return g

    def energy_terms(self, V_ext: torch.Tensor | None) -> torch.Tensor:
        """(kinetic, v_ext, v_nl, hartree, exchange) as a float64 CUDA tensor."""
        terms = torch.empty(5, dtype=torch.float64, device=_lib.require_cuda())
        _lib.call("gato_op_energy_terms", self.handle, C.c_void_p(V_ext.data_ptr() if V_ext is not None else None),
                  C.c_void_p(terms.data_ptr()), C.c_void_p(_lib.stream()))
        return terms


def _native_nl(V_nl_apply, grid: Grid3D, dtype):
    """The device operator for an HGH closure, or None for a generic callable."""
    if V_nl_apply is None or not isinstance(V_nl_apply, HGHNonlocal):
        return None
    if V_nl_apply.dtype == dtype and V_nl_apply.grid == grid:
        return V_nl_apply
    return nonlocal_for(V_nl_apply.nuclei, V_nl_apply.elements, grid, dtype)


def _density_fields(fields: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    n = fields.shape[0]
    if out is None:
        out = torch.empty(fields.shape[1:], dtype=fields.dtype, device=fields.device)
    _lib.call("gato_density", _lib.dtype_code(fields), C.c_void_p(fields.data_ptr()), n, out.numel(),
              C.c_void_p(out.data_ptr()), C.c_void_p(_lib.stream()))
    return out


def _density(orbitals) -> torch.Tensor:
    """rho = 2 sum_i |phi_i|^2 (scf.py:61-63); orbitals (N, N, N, n)."""
    return _density_fields(to_fields(orbitals))


def exchange_apply(psi, orbitals, grid: Grid3D, epsilon: float | None = None) -> torch.Tensor:
    """K psi = sum_j phi_j J[phi_j psi] (scf.py:66-85)."""
    psi = as_field(psi)
    fields = to_fields(orbitals, psi.dtype)
    eps = grid.h / 2 if epsilon is None else epsilon
    out = torch.zeros_like(psi)
    return get_plan(grid.N, grid.h, eps, psi.dtype).exchange_into(psi, fields, out, 1.0)


@dataclass(frozen=True, eq=False)
class RHFFock:
    """Closed-shell Fock operator (scf.py:114-158); duck-types as a Hamiltonian."""

    grid: Grid3D
    V_ext: torch.Tensor
    orbitals: torch.Tensor
    V_H: torch.Tensor | None = None
    boundary: str = "dirichlet"
    order: int = 4
    epsilon: float | None = None
    V_nl_apply: Callable | None = None

    def _eps(self) -> float:
        return self.grid.h / 2 if self.epsilon is None else self.epsilon

    def density(self) -> torch.Tensor:
        return _density(self.orbitals)

    def hartree(self) -> torch.Tensor:
        if self.V_H is not None:
            return as_field(self.V_H)
        return hartree_potential(self.density(), self.grid, epsilon=self.epsilon)

    def _gato_operator(self, dtype, allow_generic: bool = False):
        cache = self.__dict__.get("_ops")
        if cache is None:
            cache = {}
            object.__setattr__(self, "_ops", cache)
        if dtype in cache:
            return cache[dtype]
        nl = _native_nl(self.V_nl_apply, self.grid, dtype)
        if self.V_nl_apply is not None and nl is None and not allow_generic:
            return None   # generic V_nl callable: Lanczos takes the Python-matvec path
        fields = to_fields(self.orbitals, dtype)
        op = Operator(self.grid, dtype, self.order, self.boundary)
        V_tot = torch.empty(self.grid.shape, dtype=dtype, device=fields.device)
        Vx, Vh = as_field(self.V_ext, dtype), as_field(self.hartree(), dtype)
        _lib.call("gato_axpby", _lib.dtype_code(dtype), C.c_void_p(Vx.data_ptr()), C.c_void_p(Vh.data_ptr()),
                  C.c_void_p(V_tot.data_ptr()), V_tot.numel(), 1.0, 1.0, C.c_void_p(_lib.stream()))
        op.set_potential(V_tot)
        op.set_nonlocal(nl)
        op.set_exchange(get_plan(self.grid.N, self.grid.h, self._eps(), dtype,
                                 pair_fields(fields.shape[0])), fields)
        cache[dtype] = op
        return op

    def apply(self, psi) -> torch.Tensor:
        """F psi = T psi + V_ext psi + V_nl psi + V_H psi - K psi (scf.py:88-111)."""
        psi = as_field(psi)
        op = self._gato_operator(psi.dtype, allow_generic=True)
        out = op.apply(psi)
        if self.V_nl_apply is not None and _native_nl(self.V_nl_apply, self.grid, psi.dtype) is None:
            out = out + as_field(self.V_nl_apply(psi), psi.dtype)
        return out

    def apply_block(self) -> torch.Tensor:
        """F phi_i for all occupied orbitals, (n, N, N, N), sharing pair potentials."""
        dtype = to_fields(self.orbitals).dtype
        return self._gato_operator(dtype, allow_generic=True).apply_block()


@dataclass(frozen=True)
class RHFEnergyTerms:
    """scf.py:165-191; 0-d float64 tensors, one-body terms include the factor 2."""

    kinetic: torch.Tensor
    v_ext: torch.Tensor
    v_nl: torch.Tensor
    hartree: torch.Tensor
    exchange: torch.Tensor

    @property
    def one_body(self):
        return self.kinetic + self.v_ext + self.v_nl

    @property
    def total(self):
        return self.kinetic + self.v_ext + self.v_nl + self.hartree + self.exchange


def _energy_terms(fields, V_ext, grid, boundary, order, eps, V_nl_apply, op=None) -> torch.Tensor:
    dtype = fields.dtype
    nl = _native_nl(V_nl_apply, grid, dtype)
    if op is None:
        op = Operator(grid, dtype, order, boundary)
    op.set_nonlocal(nl)
    op.set_exchange(get_plan(grid.N, grid.h, eps, dtype, pair_fields(fields.shape[0])), fields)
    terms = op.energy_terms(as_field(V_ext, dtype) if V_ext is not None else None)
    if V_nl_apply is not None and nl is None:
        vnl = sum(inner_product(fields[i], as_field(V_nl_apply(fields[i]), dtype), grid) for i in
                  range(fields.shape[0]))
        terms = terms.clone()
        terms[2] = 2.0 * vnl
    return terms


def decompose_rhf_energy(orbitals, V_ext, grid: Grid3D, *, boundary: str = "dirichlet", order: int = 4,
                         epsilon: float | None = None, V_nl_apply=None) -> RHFEnergyTerms:
    """Every term of the closed-shell RHF energy (scf.py:194-265).

    E_x uses the pair symmetry: n(n+1)/2 Poisson solves instead of n^2.
    """
    eps = grid.h / 2 if epsilon is None else epsilon
    fields = to_fields(orbitals)
    t = _energy_terms(fields, V_ext, grid, boundary, order, eps, V_nl_apply)
    return RHFEnergyTerms(t[0], t[1], t[2], t[3], t[4])


def rhf_energy(orbitals, V_ext, grid: Grid3D, boundary: str = "dirichlet", order: int = 4,
               epsilon: float | None = None, V_nl_apply=None) -> torch.Tensor:
    """E = 2 sum_i <phi_i|h|phi_i> + E_H + E_x (scf.py:268-286)."""
    return decompose_rhf_energy(orbitals, V_ext, grid, boundary=boundary, order=order, epsilon=epsilon,
                                V_nl_apply=V_nl_apply).total


def default_initial_guess(grid: Grid3D, dtype=torch.float64) -> torch.Tensor:
    """(e^{-4r} + e^{-r}) (1 + 0.1(x+y+z) + 0.02(xy+yz+xz)) (scf.py:310-320)."""
    # evaluated on the host in FP64 and copied once (the device runs only the library's kernels)
    a = -grid.L / 2 + (torch.arange(grid.N, dtype=torch.float64) + 0.5) * grid.h
    X, Y, Z = torch.meshgrid(a, a, a, indexing="ij")
    r = torch.sqrt(X * X + Y * Y + Z * Z + 1e-6)
    psi0 = (torch.exp(-4.0 * r) + torch.exp(-r)) * (1.0 + 0.1 * (X + Y + Z) + 0.02 * (X * Y + Y * Z + X * Z))
    return as_field(psi0, dtype)


def _default_initial_orbitals(V_ext, grid: Grid3D, n_occ: int, boundary: str, order: int,
                              lanczos_iters: int, dtype=torch.float64, reorth_passes: int = 1):
    """Core-Hamiltonian guess (scf.py:289-322); returns (n, N, N, N) fields."""
    H_core = Hamiltonian(grid, as_field(V_ext, dtype), boundary, order)
    res = lanczos(H_core, default_initial_guess(grid, dtype), n_iters=lanczos_iters,
                  n_eigenstates=n_occ, reorth_passes=reorth_passes)
    return res.fields


@dataclass
class SCFResult:
    orbitals: torch.Tensor            # (N, N, N, n_occ) view of field-major storage
    energy: float
    orbital_energies: torch.Tensor    # (n_occ,)
    n_iters: int
    converged: bool
    energy_history: list = field(default_factory=list)
    terms: torch.Tensor | None = None  # last (kinetic, v_ext, v_nl, hartree, exchange)


def _total(terms: torch.Tensor) -> float:
    """Sum of the five energy terms, read back and added on the host (exactly rounded)."""
    return math.fsum(terms.tolist())


def scf_rhf(V_ext, grid: Grid3D, n_occ: int, *, initial_orbitals=None, max_iters: int = 50,
            tol: float = 1e-6, mixing: float = 1.0, boundary: str = "dirichlet", order: int = 4,
            lanczos_iters: int | None = None, epsilon: float | None = None, V_nl_apply=None,
            precision: str = "fp64", reorth_passes: int = 1) -> SCFResult:
    """Closed-shell RHF SCF loop (scf.py:335-444).

    Each iteration: V_H from the mixed density, Lanczos on the Fock operator
    (seeded with the sum of the current orbitals), linear density mixing,
    the energy of the new orbitals, and the |E_k - E_{k-1}| < tol test in FP64
    on the host. Everything between the two host reads runs on the device.

    With ``precision="mixed"`` the Fock operator, its exchange and the
    eigensolve run on FP32 fields; the density, the mixing and V_H run in FP64
    on an FP64 copy of the new orbitals. An FP32 Hartree solve carries a
    relative error near 1e-7 in E_H (about 2e-6 Ha for water), larger than the
    1e-6 Ha agreement the two precisions are held to, so the energy is FP64
    wherever it decides anything: the FP32 energy terms serve only while
    |E_k - E_{k-1}| > max(1e3 tol, 1e-4); from the first iterate below that,
    every energy (and every convergence test) is FP64, and the returned energy
    is always an FP64 evaluation.
    """
    dtype = precision_dtype(precision)
    mixed = dtype != torch.float64
    f64 = torch.float64
    dev = _lib.require_cuda()
    dc = _lib.dtype_code(dtype)
    eps = grid.h / 2 if epsilon is None else epsilon
    m = default_krylov_dim(grid.N, n_occ) if lanczos_iters is None else int(lanczos_iters)
    K = min(n_occ, m)
    V_ext64 = as_field(V_ext, f64)
    V_ext = as_field(V_ext, dtype)
    nl = _native_nl(V_nl_apply, grid, dtype)
    generic_nl = V_nl_apply is not None and nl is None
    plan = get_plan(grid.N, grid.h, eps, dtype, pair_fields(n_occ))
    plan64 = get_plan(grid.N, grid.h, eps, f64, pair_fields(n_occ))
    if initial_orbitals is None:
        orb = _default_initial_orbitals(V_ext, grid, n_occ, boundary, order, m, dtype, reorth_passes)
    else:
        orb = to_fields(initial_orbitals, dtype)
    orb = orb.contiguous()
    n3 = grid.N ** 3
    s = lambda: C.c_void_p(_lib.stream())   # noqa: E731
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def convert(src, dst):
        _lib.call("gato_convert", _lib.dtype_code(src), P(src), _lib.dtype_code(dst), P(dst), src.numel(), s())
        return dst

    orb64 = convert(orb, torch.empty(orb.shape, dtype=f64, device=dev)) if mixed else orb
    rho = _density_fields(orb64)
    rho_new = torch.empty_like(rho)
    V_H = torch.empty_like(rho)
    V_tot64 = torch.empty_like(rho)
    V_tot = torch.empty(grid.shape, dtype=dtype, device=dev) if mixed else V_tot64
    seed = torch.empty(grid.shape, dtype=dtype, device=dev)
    krylov = torch.empty((m + 1,) + grid.shape, dtype=dtype, device=dev)
    bufs = [torch.empty((K,) + grid.shape, dtype=dtype, device=dev) for _ in range(2)]
    op = Operator(grid, dtype, order, boundary)
    op.set_nonlocal(nl)
    op64 = Operator(grid, f64, order, boundary) if mixed else op
    buf64 = torch.empty((K,) + grid.shape, dtype=f64, device=dev) if mixed else None
    history: list[float] = []
    E_prev = float("inf")
    E = float("inf")
    # Mixed precision: the FP32 energy terms carry ~1e-7 relative noise (up to ~1e-5 Ha on
    # small grids), harmless while the energy still moves by more than `switch` per iteration;
    # below that every energy (and so every convergence test) is FP64. The plain path is FP64
    # throughout.
    energy64 = not mixed
    switch = max(1e3 * tol, 1e-4)
    orbital_energies = torch.zeros(n_occ, dtype=f64).to(dev)   # a copy, no device kernel
    converged = False
    terms = None
    it = 0
    for it in range(1, max_iters + 1):
        plan64.potential(rho, out=V_H)
        _lib.call("gato_axpby", _lib.F64, P(V_ext64), P(V_H), P(V_tot64), n3, 1.0, 1.0, s())
        if mixed:
            convert(V_tot64, V_tot)
        op.set_potential(V_tot)
        op.set_exchange(plan, orb)
        _lib.call("gato_field_sum", dc, P(orb), orb.shape[0], n3, P(seed), s())
        new = bufs[it % 2]
        if generic_nl:
            fock = RHFFock(grid, V_ext, from_fields(orb), V_H, boundary, order, eps, V_nl_apply)
            res = lanczos(fock, seed, n_iters=m, n_eigenstates=n_occ, krylov=krylov, out=new,
                          reorth_passes=reorth_passes)
        else:
            res = lanczos(_Bound(grid, op), seed, n_iters=m, n_eigenstates=n_occ, krylov=krylov, out=new,
                          reorth_passes=reorth_passes)
        orbital_energies = res.eigenvalues
        orb = new
        orb64 = convert(orb, buf64[: orb.shape[0]]) if mixed else orb
        _density_fields(orb64, rho_new)
        _lib.call("gato_mix", _lib.F64, P(rho), P(rho_new), n3, float(mixing), s())
        if energy64:
            terms = _energy_terms(orb64, V_ext64, grid, boundary, order, eps, V_nl_apply, op=op64)
            E = _total(terms)
        else:
            terms = _energy_terms(orb, V_ext, grid, boundary, order, eps, V_nl_apply, op=op)
            E = _total(terms)
            if abs(E - E_prev) < switch:
                # close to the stop: from here on every energy is FP64, starting with this iterate
                energy64 = True
                terms = _energy_terms(orb64, V_ext64, grid, boundary, order, eps, V_nl_apply, op=op64)
                E = _total(terms)
                history.append(E)
                E_prev = E
                continue
        history.append(E)
        if energy64 and abs(E - E_prev) < tol:
            converged = True
            break
        E_prev = E
    if not energy64:
        # max_iters reached on FP32 energies: the reported energy is still an FP64 evaluation
        terms = _energy_terms(orb64, V_ext64, grid, boundary, order, eps, V_nl_apply, op=op64)
        E = _total(terms)
    return SCFResult(from_fields(orb), E, orbital_energies, it, converged, history, terms)


class _Bound:
    """Adapter presenting an already-configured Operator to ``lanczos``."""

    def __init__(self, grid: Grid3D, op: Operator):
        self.grid, self._op = grid, op

    def _gato_operator(self, dtype):
        return self._op if dtype == self._op.dtype else None

    def apply(self, psi):
        return self._op.apply(as_field(psi, self._op.dtype))
