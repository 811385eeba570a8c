"""Autotuner for the pair-solve pipeline.

Times a caller-supplied step (e.g. one block Fock apply) for each candidate
(fields per launch group, FFT engine) of a Poisson plan with CUDA events and
keeps the fastest. Fewer fields per group keep each field's spectral
intermediates (N M^2 complex values) resident in L2 between the passes;
more fields per group give larger launches. Results are cached per
(N, dtype, workload key) for the life of the process.
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
