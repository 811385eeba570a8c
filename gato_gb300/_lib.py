"""ctypes binding of libgato_cuda (the C ABI declared in include/gato.h).

The library is the only compute path: if it is missing or no CUDA device is
present, every operation raises instead of falling back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import torch

from . import build as _build

GATO_OK = 0
GATO_EBADARG = -1
GATO_ECUDA = -2
GATO_ETIMEOUT = -3
GATO_ENOMEM = -4
GATO_EUNSUPPORTED = -5
GATO_EKEY = -6

F64, F32 = 0, 1
DIRICHLET, PERIODIC = 0, 1

_lock = threading.Lock()
_lib = None

vp, i32, i64, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_double
P_f64 = C.POINTER(C.c_double)
P_i32 = C.POINTER(C.c_int)

# name -> argument types (all return int status)
_SIGS = {
    "gato_version": [],
    "gato_last_error": [C.c_char_p, C.c_size_t],
    "gato_device_status": [P_i32, vp],
    "gato_dot": [i32, vp, vp, i64, f64, vp, vp],
    "gato_dot_noalloc": [i32, vp, vp, i64, f64, vp, vp],
    "gato_normalize": [i32, vp, i64, vp, vp],
    "gato_stencil_apply": [i32, vp, vp, vp, i32, i32, i32, i32, f64, i32, i32, vp, f64, vp],
    "gato_stencil_tune": [i32],
    "gato_softened_coulomb": [i32, vp, i32, f64, i32, P_f64, P_f64, f64, vp],
    "gato_hgh_local": [i32, vp, i32, f64, i32, P_f64, P_f64, P_f64, P_f64, vp],
    "gato_nonlocal_create": [i32, i32, f64, i32, P_f64, P_i32, P_i32, P_f64, P_i32, P_f64, f64,
                             C.POINTER(vp)],
    "gato_nonlocal_destroy": [vp],
    "gato_nonlocal_apply": [vp, vp, vp, i32, vp],
    "gato_nonlocal_energy": [vp, vp, i32, vp, vp],
    "gato_poisson_create": [i32, i32, f64, f64, i32, C.POINTER(vp), vp],
    "gato_poisson_destroy": [vp],
    "gato_hartree_potential": [vp, vp, vp, vp],
    "gato_hartree_energy": [vp, vp, vp, vp],
    "gato_poisson_stage": [vp, i32, i32, vp],
    "gato_poisson_tune": [vp, i32, i32],
    "gato_op_tune": [vp, i32],
    "gato_op_overlap": [vp, i32],
    "gato_density": [i32, vp, i32, i64, vp, vp],
    "gato_mix": [i32, vp, vp, i64, f64, vp],
    "gato_exchange_apply": [vp, vp, vp, i32, vp, f64, vp],
    "gato_axpby": [i32, vp, vp, vp, i64, f64, f64, vp],
    "gato_field_sum": [i32, vp, i32, i64, vp, vp],
    "gato_convert": [i32, vp, i32, vp, i64, vp],
    "gato_dot_weighted": [i32, vp, vp, vp, i64, f64, vp, vp],
    "gato_imag_time": [i32, vp, vp, i32, f64, i32, i32, f64, i32, i32, vp, vp],
    "gato_radial_density": [i32, vp, vp, i32, f64, P_f64, i32, vp, vp],
    "gato_op_create": [i32, i32, f64, i32, i32, C.POINTER(vp)],
    "gato_op_destroy": [vp],
    "gato_op_set_potential": [vp, vp],
    "gato_op_set_nonlocal": [vp, vp],
    "gato_op_set_exchange": [vp, vp, vp, i32],
    "gato_op_apply": [vp, vp, vp, vp],
    "gato_op_apply_block": [vp, vp, vp],
    "gato_op_energy_terms": [vp, vp, vp, vp],
    "gato_lanczos": [vp, vp, i32, i32, f64, i32, vp, vp, vp, vp, vp, vp, vp],
    "gato_lanczos_begin": [i32, i64, f64, vp, vp, i32, i32, vp],
    "gato_lanczos_step": [i32, i64, f64, vp, i32, i32, i32, i32, vp, vp, vp],
    "gato_lanczos_tune": [i32],
    "gato_lanczos_finish": [i32, i64, vp, i32, i32, f64, vp, vp, vp, vp, vp, vp],
    "gato_hgh_local_grad": [i32, vp, i32, f64, i32, P_f64, P_f64, P_f64, P_f64, P_f64, vp],
    "gato_nonlocal_grad": [vp, vp, i32, P_f64, vp],
    "gato_softened_coulomb_grad": [i32, vp, i32, f64, i32, P_f64, P_f64, f64, P_f64, vp],
}


def library_path() -> str:
    return _build.LIB


def lib():
    """Load (building first if needed) libgato_cuda.so; raise if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) or not _build.up_to_date():
            _build.build()
        L = C.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.gato_launch_count.argtypes = []
        L.gato_launch_count.restype = C.c_longlong
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().gato_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    """Map a gato status to the exception the reference raises."""
    if status == GATO_OK:
        return
    msg = last_error()
    if status == GATO_EBADARG:
        raise ValueError(msg)
    if status == GATO_EUNSUPPORTED:
        raise NotImplementedError(msg)
    if status == GATO_EKEY:
        raise KeyError(msg)
    if status == GATO_ENOMEM:
        raise MemoryError(msg)
    if status == GATO_ETIMEOUT:
        raise TimeoutError(msg)
    raise RuntimeError(f"libgato_cuda error {status}: {msg}")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("gato_gb300 needs a CUDA device (GB300); there is no CPU path")
    lib()
    return torch.device("cuda", torch.cuda.current_device())


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def dtype_code(t) -> int:
    dt = t.dtype if isinstance(t, torch.Tensor) else t
    if dt == torch.float64:
        return F64
    if dt == torch.float32:
        return F32
    raise TypeError(f"unsupported dtype {dt}; expected float64 or float32")


def boundary_code(boundary: str) -> int:
    if boundary == "dirichlet":
        return DIRICHLET
    if boundary == "periodic":
        return PERIODIC
    raise ValueError(f"Unknown boundary {boundary!r}; expected 'dirichlet' or 'periodic'.")


def dbl_array(values):
    vals = [float(v) for v in values]
    return (C.c_double * max(len(vals), 1))(*vals)


def int_array(values):
    vals = [int(v) for v in values]
    return (C.c_int * max(len(vals), 1))(*vals)


def launch_count() -> int:
    return int(lib().gato_launch_count())


def device_status() -> int:
    v = C.c_int(0)
    call("gato_device_status", C.byref(v), C.c_void_p(stream()))
    return v.value
