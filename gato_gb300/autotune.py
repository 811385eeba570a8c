"""Autotuner for the pair-solve pipeline and the stencil tile shape.

Times a caller-supplied step (e.g. one block Fock apply) for each candidate
(fields per launch group, FFT engine) of a Poisson plan with CUDA events and
keeps the fastest. Fewer fields per group keep each field's spectral
intermediates (N M^2 complex values) resident in L2 between the passes;
more fields per group give larger launches. The stencil's TMA kernel is tuned
the same way over its tile shapes (rows per thread: 2 or 4). Results are
cached per (N, dtype, workload key) for the life of the process.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

_CACHE: dict = {}


def set_plan(plan, group: int, engine: int = 0) -> None:
    _lib.call("gato_poisson_tune", plan.handle, int(group), int(engine))


def tune_plan(plan, step, key=None, groups=None, reps: int = 3, engines=(0,)) -> dict:
    """Pick the fastest (group, engine) for `step()` and apply it to `plan`."""
    key = (plan.N, plan.dtype, plan.max_fields, key)
    if key in _CACHE:
        best = _CACHE[key]
        set_plan(plan, best["group"], best["engine"])
        return best
    if groups is None:
        groups = sorted({1, 2, 3, plan.max_fields} & set(range(1, plan.max_fields + 1)))
    results = []
    for engine in engines:
        for g in groups:
            set_plan(plan, g, engine)
            step()
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                step()
                b.record()
                b.synchronize()
                ts.append(a.elapsed_time(b))
            results.append({"group": g, "engine": engine, "ms": min(ts)})
    best = min(results, key=lambda r: r["ms"])
    best = dict(best, candidates=results)
    set_plan(plan, best["group"], best["engine"])
    _CACHE[key] = best
    return best


def _time(step, reps: int) -> float:
    step()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        step()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return min(ts)


def tune_stencil(step, key=None, reps: int = 5) -> dict:
    """Pick the stencil tile shape (rows per thread 2 or 4) that runs `step()` fastest.

    The choice is process-wide (one knob for every stencil launch)."""
    key = ("stencil", key)
    if key in _CACHE:
        best = _CACHE[key]
        _lib.call("gato_stencil_tune", best["rows"])
        return best
    results = []
    for rows in (2, 4):
        _lib.call("gato_stencil_tune", rows)
        results.append({"rows": rows, "ms": _time(step, reps)})
    best = min(results, key=lambda r: r["ms"])
    best = dict(best, candidates=results)
    _lib.call("gato_stencil_tune", best["rows"])
    _CACHE[key] = best
    return best


def tune_block_epilogue(op, step, key=None, reps: int = 5) -> dict:
    """Pick the block-apply epilogue of operator `op` that runs `step()` fastest:
    1 = the J_ij fields and one pair pass, 2 = accumulation in the z-inverse epilogue."""
    key = ("block_epi", op.grid.N, op.dtype, key)
    if key in _CACHE:
        best = _CACHE[key]
        op.tune(best["epilogue"])
        return best
    results = []
    for epi in (1, 2):
        op.tune(epi)
        results.append({"epilogue": epi, "ms": _time(step, reps)})
    best = min(results, key=lambda r: r["ms"])
    best = dict(best, candidates=results)
    op.tune(best["epilogue"])
    _CACHE[key] = best
    return best
