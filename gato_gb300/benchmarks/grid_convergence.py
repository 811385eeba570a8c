"""Convergence of GPU RHF results with grid spacing and box size.

Reference counterpart: benchmarks/grid_convergence.py (a sweep harness over the
water and HCl drivers). This module is organised around a declarative list of
sweep points instead of per-molecule adapter classes:

* a **study** is a list of ``SweepPoint(molecule, N, L, task)`` records,
  built by ``spacing_study`` (N varies at fixed L), ``box_study`` (L varies at
  a held spacing, N = nearest even L / h) or ``relax_study`` (a geometry
  relaxation per N);
* ``run_study`` evaluates every point with the package's own SCF (and
  optimiser) and returns JSON-ready records, one per point;
* ``extrapolate`` fits y(x) = y_inf + C x^p by **variable projection**
  (Golub and Pereyra, SIAM J. Numer. Anal. 10, 1973): for a fixed exponent the
  model is linear in (y_inf, C), which linear least squares eliminates, and
  the remaining one-dimensional residual is minimised over p with Brent's
  bounded method.

The command line prints the records and fits as one JSON document::

    python -m gato_gb300.benchmarks.grid_convergence water spacing --N 32 40 48 --L 12
    python -m gato_gb300.benchmarks.grid_convergence hcl box --sides 8 9 10 --h 0.25 --out box.json
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from dataclasses import asdict, dataclass

import numpy as np

from ..geometry import bond_angle, bond_length
from ..grid import Grid3D
from ..physics import hcl, water

# molecule name -> (starting geometry, HGH elements, single-point solver, relaxation driver)
MOLECULES = {
    "water": (water.water_initial_geometry, water.water_hgh_elements, water.solve_rhf_at_geometry,
              water.optimize_water_geometry),
    "hcl": (hcl.hcl_initial_geometry, hcl.hcl_hgh_elements, hcl.solve_rhf_at_geometry,
            hcl.optimize_geometry),
}


@dataclass(frozen=True)
class SweepPoint:
    molecule: str
    N: int
    L: float
    task: str = "energy"    # "energy": one SCF; "relax": geometry relaxation then its energy

    @property
    def h(self) -> float:
        return self.L / self.N


def spacing_study(molecule: str, Ns, L: float) -> list[SweepPoint]:
    return [SweepPoint(molecule, int(n), float(L)) for n in Ns]


def box_study(molecule: str, sides, h: float) -> list[SweepPoint]:
    """One point per box side, N the even integer nearest to L / h."""
    return [SweepPoint(molecule, 2 * max(1, int(round(s / h / 2.0))), float(s)) for s in sides]


def relax_study(molecule: str, Ns, L: float) -> list[SweepPoint]:
    return [SweepPoint(molecule, int(n), float(L), task="relax") for n in Ns]


def _shape(nuclei) -> dict:
    """Bond length of nuclei 0-1 and, for three nuclei, the angle at nucleus 0 (degrees)."""
    out = {"R": float(bond_length(nuclei, 0, 1))}
    if nuclei.n == 3:
        out["angle"] = math.degrees(float(bond_angle(nuclei, 1, 0, 2)))
    return out


def evaluate(pt: SweepPoint, *, order: int = 4, precision: str = "mixed", max_scf: int = 60,
             relax_steps: int = 20, relax_lr: float = 0.04) -> dict:
    """One record: the point, its energy, SCF outcome and wall time (and the relaxed shape)."""
    geometry, elements, solve, relax = MOLECULES[pt.molecule]
    grid = Grid3D(N=pt.N, L=pt.L)
    t0 = time.perf_counter()
    if pt.task == "energy":
        res = solve(geometry(), elements(), grid, max_iters=max_scf, order=order, precision=precision)
        rec = {"E": float(res.energy), "scf_iters": int(res.n_iters), "converged": bool(res.converged)}
    elif pt.task == "relax":
        opt = relax(geometry(), elements(), grid, geom_steps=relax_steps, learning_rate=relax_lr,
                    scf_max_iters=max_scf, order=order, verbose=False, precision=precision)
        fin = opt.final
        rec = {"E": float(fin.energy), "scf_iters": int(fin.n_iters), "converged": bool(fin.converged),
               **_shape(fin.nuclei)}
    else:
        raise ValueError(f"unknown task {pt.task!r}")
    return {**asdict(pt), "h": pt.h, **rec, "seconds": time.perf_counter() - t0}


def run_study(points, log=None, **kw) -> list[dict]:
    """Evaluate every point in order; ``log`` (a file) gets one line per finished point."""
    records = []
    for pt in points:
        rec = evaluate(pt, **kw)
        records.append(rec)
        if log is not None:
            print(f"[{pt.molecule} {pt.task} N={pt.N} L={pt.L:g} h={pt.h:.5f}] E={rec['E']:+.8f} "
                  f"scf={rec['scf_iters']} conv={rec['converged']} {rec['seconds']:.1f}s", file=log, flush=True)
    return records


def extrapolate(xs, ys, p_bounds=(0.5, 6.0)) -> dict | None:
    """Variable-projection fit of y = y_inf + C x^p; None with fewer than three points.

    For fixed p, (y_inf, C) solve a two-column linear least-squares problem;
    p minimises the resulting residual norm (Brent, bounded). The residual is
    also compared at the two bounds, so a monotone residual returns the
    better bound rather than an interior stationary point.
    """
    from scipy.optimize import minimize_scalar

    x = np.asarray(xs, dtype=float)
    y = np.asarray(ys, dtype=float)
    if x.size < 3:
        return None

    def solve_linear(p):
        A = np.column_stack([np.ones_like(x), x ** p])
        coef, *_ = np.linalg.lstsq(A, y, rcond=None)
        r = y - A @ coef
        return coef, float(np.sqrt(np.mean(r * r)))

    opt = minimize_scalar(lambda p: solve_linear(p)[1], bounds=p_bounds, method="bounded",
                          options={"xatol": 1e-12})
    cands = [float(opt.x), float(p_bounds[0]), float(p_bounds[1])]
    p = min(cands, key=lambda q: solve_linear(q)[1])
    coef, rms = solve_linear(p)
    return {"y_inf": float(coef[0]), "C": float(coef[1]), "p": p, "rms": rms, "points": int(x.size)}


def summarise(study: str, records: list[dict]) -> dict:
    """The fits a study supports, over the points whose SCF converged.

    spacing: E against h. box: E against 1/L, plus the spread of the spacing
    actually used (a box study holds h only as far as L / N allows). relax:
    E, R (and the angle) against h.
    """
    ok = [r for r in records if r["converged"]]
    out: dict = {"study": study, "points": len(records), "converged": len(ok)}
    hs = [r["h"] for r in ok]
    if study == "spacing":
        out["E_vs_h"] = extrapolate(hs, [r["E"] for r in ok])
    elif study == "box":
        out["E_vs_inv_L"] = extrapolate([1.0 / r["L"] for r in ok], [r["E"] for r in ok])
        out["h_spread"] = (max(hs) - min(hs)) if hs else None
    elif study == "relax":
        for key in ("E", "R", "angle"):
            if ok and key in ok[0]:
                out[f"{key}_vs_h"] = extrapolate(hs, [r[key] for r in ok])
    return out


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description="grid and box convergence of GPU RHF energies")
    ap.add_argument("molecule", choices=sorted(MOLECULES))
    ap.add_argument("study", choices=["spacing", "box", "relax"])
    ap.add_argument("--N", type=int, nargs="+", default=[32, 40, 48, 56, 64],
                    help="grid points per axis (spacing and relax studies)")
    ap.add_argument("--L", type=float, default=12.0, help="box side in bohr (spacing and relax studies)")
    ap.add_argument("--sides", type=float, nargs="+", default=[10.0, 12.0, 14.0, 16.0],
                    help="box sides in bohr (box study)")
    ap.add_argument("--h", type=float, default=0.25, help="held grid spacing in bohr (box study)")
    ap.add_argument("--order", type=int, choices=[2, 4], default=4)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--max-scf", type=int, default=60)
    ap.add_argument("--relax-steps", type=int, default=20)
    ap.add_argument("--relax-lr", type=float, default=0.04)
    ap.add_argument("--out", default=None, help="write the JSON document here instead of stdout")
    ap.add_argument("--quiet", action="store_true", help="no per-point progress lines on stderr")
    a = ap.parse_args(argv)
    if a.study == "spacing":
        points = spacing_study(a.molecule, a.N, a.L)
    elif a.study == "box":
        points = box_study(a.molecule, a.sides, a.h)
    else:
        points = relax_study(a.molecule, a.N, a.L)
    records = run_study(points, log=None if a.quiet else sys.stderr, order=a.order, precision=a.precision,
                        max_scf=a.max_scf, relax_steps=a.relax_steps, relax_lr=a.relax_lr)
    doc = {"records": records, "summary": summarise(a.study, records)}
    text = json.dumps(doc, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text + "\n")
    else:
        print(text)
    return doc


if __name__ == "__main__":
    main()
