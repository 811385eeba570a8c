"""Matrix-free Lanczos with full reorthogonalisation (reference: lanczos.py:1-206).

For the library's own operators (``Hamiltonian``, ``RHFFock``) the whole
m-step loop, the tridiagonal eigensolve and the Ritz reconstruction run on
the device in one call with no host synchronisation; any other object with
``.grid`` and ``.apply`` (the reference's duck-typed contract) gets the same
device reorthogonalisation around its own Python matvec.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from .. import _lib
from ..grid import as_field


@dataclass
class LanczosResult:
    eigenvalues: torch.Tensor   # (K,) float64, ascending
    eigenstates: torch.Tensor   # (*grid.shape, K) view of field-major storage
    n_iters: int
    converged: bool             # True if any beta fell below tol
    alphas: torch.Tensor | None = None
    betas: torch.Tensor | None = None

    @property
    def fields(self) -> torch.Tensor:
        """The Ritz vectors as a contiguous (K, N, N, N) block."""
        return self.eigenstates.permute(3, 0, 1, 2)


def default_krylov_dim(N: int, n_eigenstates: int = 1) -> int:
    """max(24 n + 24, 5N/4) (lanczos.py:49-107)."""
    return max(24 * n_eigenstates + 24, (5 * N) // 4)


def lanczos(H, psi0, n_iters: int = 80, n_eigenstates: int = 4, tol: float = 1e-10, *,
            reorth_passes: int = 1, krylov: torch.Tensor | None = None,
            out: torch.Tensor | None = None) -> LanczosResult:
    """Lowest ``n_eigenstates`` eigenpairs of H from ``n_iters`` Lanczos steps.

    The dtype of ``psi0`` selects the path: float64 (plain) or float32
    (mixed: FP32 basis and matvecs, FP64 coefficients and eigensolve).
    ``krylov`` ((n_iters+1, N, N, N)) and ``out`` ((K, N, N, N)) may be
    passed to reuse buffers.
    """
    psi0 = as_field(psi0)
    if torch.is_complex(psi0):
        raise TypeError("lanczos: complex start vectors are not supported")
    dtype, shape = psi0.dtype, tuple(psi0.shape)
    dc = _lib.dtype_code(dtype)
    m = int(n_iters)
    K = min(int(n_eigenstates), m)
    n = psi0.numel()
    dev = psi0.device
    if krylov is None:
        krylov = torch.empty((m + 1,) + shape, dtype=dtype, device=dev)
    if out is None:
        out = torch.empty((K,) + shape, dtype=dtype, device=dev)
    alphas = torch.empty(m, dtype=torch.float64, device=dev)
    betas = torch.empty(m, dtype=torch.float64, device=dev)
    evals = torch.empty(K, dtype=torch.float64, device=dev)
    flag = torch.empty(1, dtype=torch.int32, device=dev)   # always written by the eigensolve
    s = C.c_void_p(_lib.stream())
    op = H._gato_operator(dtype) if hasattr(H, "_gato_operator") else None
    if op is not None:
        _lib.call("gato_lanczos", op.handle, C.c_void_p(psi0.data_ptr()), m, K, float(tol),
                  reorth_passes, C.c_void_p(krylov.data_ptr()), C.c_void_p(evals.data_ptr()),
                  C.c_void_p(out.data_ptr()), C.c_void_p(alphas.data_ptr()),
                  C.c_void_p(betas.data_ptr()), C.c_void_p(flag.data_ptr()), s)
    else:
        dV = H.grid.dV
        _lib.call("gato_lanczos_begin", dc, n, dV, C.c_void_p(psi0.data_ptr()),
                  C.c_void_p(krylov.data_ptr()), m, K, s)
        for j in range(m):
            krylov[j + 1].copy_(as_field(H.apply(krylov[j]), dtype))
            _lib.call("gato_lanczos_step", dc, n, dV, C.c_void_p(krylov.data_ptr()), j, m, K,
                      reorth_passes, C.c_void_p(alphas.data_ptr()), C.c_void_p(betas.data_ptr()), s)
        _lib.call("gato_lanczos_finish", dc, n, C.c_void_p(krylov.data_ptr()), m, K, float(tol),
                  C.c_void_p(alphas.data_ptr()), C.c_void_p(betas.data_ptr()),
                  C.c_void_p(evals.data_ptr()), C.c_void_p(out.data_ptr()),
                  C.c_void_p(flag.data_ptr()), s)
    converged = bool(flag.item())
    return LanczosResult(evals, out.permute(1, 2, 3, 0), m, converged, alphas, betas)
