"""gato_dot_noalloc: the grid inner product for callers that cannot allocate.

Hosts that own all device memory through their own allocator, and threads
that must not block in cudaMalloc, cannot use gato_dot (whose partial sums
come from scratch allocated on first use). gato_dot_noalloc keeps them in a
static device array. This file calls it through the C ABI on two calls in a
row (the array keeps the previous call's contents, which must not leak into
the next result) and compares each result with gato_dot and with an FP64
NumPy sum of the same inputs; it also checks the size limit. It is named to
be collected last, and passes alone in a fresh process or after the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from gato_gb300 import _lib
    return _lib


def _dot(lib, fn, a, b, scale):
    out = torch.empty((), dtype=torch.float64, device="cuda")
    lib.call(fn, lib.dtype_code(a), C.c_void_p(a.data_ptr()),
             C.c_void_p(b.data_ptr() if b is not None else None), a.numel(), scale,
             C.c_void_p(out.data_ptr()), C.c_void_p(lib.stream()))
    return float(out)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_noalloc_dot_matches_dot_twice(lib, dtype):
    rng = np.random.default_rng(7)
    g1 = [torch.tensor(rng.standard_normal(64 ** 3), device="cuda", dtype=dtype) for _ in range(2)]
    # second call: a smaller input, so stale partials of the first call would show
    g2 = [torch.tensor(rng.standard_normal(24 ** 3 + 5), device="cuda", dtype=dtype) for _ in range(2)]
    tol = 1e-12 if dtype == torch.float64 else 1e-6
    for a, b in (g1, g2):
        a64, b64 = a.double().cpu().numpy(), b.double().cpu().numpy()
        exact = 0.125 * float(np.dot(a64, b64))
        exact_sum = float(np.sum(a64))
        ref = _dot(lib, "gato_dot", a, b, 0.125)
        got = _dot(lib, "gato_dot_noalloc", a, b, 0.125)
        assert abs(got - ref) <= tol * max(1.0, abs(ref)), (got, ref)
        # the FP32 path sums exact products in float-float: FP64-level agreement with numpy
        assert abs(got - exact) <= 1e-12 * max(1.0, abs(exact)), (got, exact)
        ref_sum = _dot(lib, "gato_dot", a, None, 1.0)
        got_sum = _dot(lib, "gato_dot_noalloc", a, None, 1.0)
        assert abs(got_sum - ref_sum) <= tol * max(1.0, abs(ref_sum))
        assert abs(got_sum - exact_sum) <= 1e-12 * max(1.0, abs(exact_sum)), (got_sum, exact_sum)


def test_noalloc_dot_rejects_oversized_input(lib):
    a = torch.ones(8, dtype=torch.float64, device="cuda")
    out = torch.empty((), dtype=torch.float64, device="cuda")
    # the size check happens before any device access, so a too-large n is safe to pass
    with pytest.raises(ValueError, match="exceeds the maximum"):
        lib.call("gato_dot_noalloc", lib.F64, C.c_void_p(a.data_ptr()), None, (1 << 27) + 1, 1.0,
                 C.c_void_p(out.data_ptr()), C.c_void_p(lib.stream()))
