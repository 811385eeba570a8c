"""Grid-convergence study for the HGH molecules (reference: benchmarks/grid_convergence.py:1-308).

A real-space result carries a resolution error (the spacing h = L/N) and a
box error (the side L). Three sweeps separate them, each finished by a fit
E(x) = E_inf + C x^p whose order p is found by a scan:

    energy    E(h) at fixed L and geometry      -> resolution error, h -> 0
    box       E(L) at fixed h (N = L / h)       -> box error, 1/L -> 0
    geometry  relaxed R, angle and E against h  -> does the geometry converge

    python -m gato_gb300.benchmarks.grid_convergence --molecule water --mode energy
    python -m gato_gb300.benchmarks.grid_convergence --molecule hcl --mode box --precision mixed

Each SCF runs on the GPU through the package's own solvers; ``--precision
mixed`` uses the FP32 Fock path with FP64 energies, which makes the larger
grids of the sweep cheap.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from ..geometry import bond_angle, bond_length
from ..grid import Grid3D
from ..physics import hcl as hcl_mod
from ..physics import water as water_mod


class WaterCase:
    name = "H2O"
    default_L = 14.0
    R0, angle0 = 1.81, 104.5   # near the relaxed geometry

    def nuclei(self):
        return water_mod.water_initial_geometry(R_OH=self.R0, angle_deg=self.angle0)

    def elements(self):
        return water_mod.water_hgh_elements()

    def solve(self, nuclei, grid, **kw):
        return water_mod.solve_rhf_at_geometry(nuclei, self.elements(), grid, **kw)

    def optimize(self, grid, **kw):
        res = water_mod.optimize_water_geometry(self.nuclei(), self.elements(), grid, verbose=False, **kw)
        n = res.final.nuclei
        return {"E": res.final.energy, "R": float(bond_length(n, 0, 1)),
                "angle": math.degrees(float(bond_angle(n, 1, 0, 2))), "converged": res.final.converged}


class HClCase:
    name = "HCl"
    default_L = 14.0
    R0 = 2.41

    def nuclei(self):
        return hcl_mod.hcl_initial_geometry(R_HCl=self.R0)

    def elements(self):
        return hcl_mod.hcl_hgh_elements()

    def solve(self, nuclei, grid, **kw):
        return hcl_mod.solve_rhf_at_geometry(nuclei, self.elements(), grid, **kw)

    def optimize(self, grid, **kw):
        kw.pop("lanczos_iters", None)
        res = hcl_mod.optimize_geometry(self.nuclei(), self.elements(), grid, verbose=False, **kw)
        n = res.final.nuclei
        return {"E": res.final.energy, "R": float(bond_length(n, 0, 1)), "angle": float("nan"),
                "converged": res.final.converged}


CASES = {"water": WaterCase, "hcl": HClCase}


def fit_power_law(xs, ys):
    """Least-squares y = y_inf + C x^p over a scan of p in [0.5, 6] (1101 points).

    For a fixed p the model is linear in (y_inf, C): one 2-column lstsq per
    candidate; the p with the smallest rms residual wins. Returns
    (y_inf, C, p, rms), all nan with fewer than three points.
    """
    x = np.asarray(xs, dtype=float)
    y = np.asarray(ys, dtype=float)
    if x.size < 3:
        return (float("nan"),) * 4
    best = None
    for p in np.linspace(0.5, 6.0, 1101):
        A = np.stack([np.ones_like(x), x ** p], axis=1)
        coef = np.linalg.lstsq(A, y, rcond=None)[0]
        rms = float(np.sqrt(np.mean((y - A @ coef) ** 2)))
        if best is None or rms < best[3]:
            best = (float(coef[0]), float(coef[1]), float(p), rms)
    return best


def _report(label, xs, ys, unit):
    y_inf, _, p, rms = fit_power_law(xs, ys)
    if math.isnan(p):
        print(f"  {label}: need >= 3 points to fit")
        return None
    print(f"  {label}: extrapolated {y_inf:+.6f} {unit}   (order p = {p:.2f}, rms resid = {rms:.2e})")
    return {"extrapolated": y_inf, "order": p, "rms": rms}


def sweep_energy(case, Ns, L, order, scf_iters, precision="fp64"):
    """E against h at fixed L and geometry."""
    print(f"{case.name}: energy vs grid spacing at fixed L = {L} a0, stencil order {order}, {precision}")
    print(f"{'N':>5} {'h (a0)':>9} {'E (Ha)':>15} {'SCF it':>7} {'conv':>6} {'time':>8}")
    rows, nuclei = [], case.nuclei()
    for N in Ns:
        grid = Grid3D(N=N, L=L)
        t0 = time.perf_counter()
        pt = case.solve(nuclei, grid, max_iters=scf_iters, order=order, precision=precision)
        dt = time.perf_counter() - t0
        print(f"{N:5d} {grid.h:9.5f} {pt.energy:+15.8f} {pt.n_iters:7d} {str(pt.converged):>6} {dt:7.2f}s",
              flush=True)
        rows.append({"N": N, "h": grid.h, "E": pt.energy, "iters": pt.n_iters, "converged": pt.converged,
                     "seconds": dt})
        if not pt.converged:
            print("      ^ left out of the fit: SCF did not converge")
    print()
    ok = [r for r in rows if r["converged"]]
    fit = _report("E(h -> 0)", [r["h"] for r in ok], [r["E"] for r in ok], "Ha")
    return {"rows": rows, "fit": fit}


def sweep_box(case, Ls, target_h, order, scf_iters, precision="fp64"):
    """E against L at (nearly) fixed h: N = L / h rounded to an even integer.

    The achieved h is printed and a drift in h is reported, since dE/dh near
    h = 0.175 is about 1.6 Ha per bohr and a 1.5% drift in h swamps the box
    effect; pick target_h so that every L / target_h is an integer.
    """
    print(f"{case.name}: energy vs box size at fixed h ~ {target_h} a0, stencil order {order}, {precision}")
    print(f"{'L':>6} {'N':>5} {'h (a0)':>9} {'E (Ha)':>15} {'SCF it':>7} {'conv':>6} {'time':>8}")
    rows, nuclei = [], case.nuclei()
    for L in Ls:
        N = int(round(L / target_h / 2)) * 2
        grid = Grid3D(N=N, L=L)
        t0 = time.perf_counter()
        pt = case.solve(nuclei, grid, max_iters=scf_iters, order=order, precision=precision)
        dt = time.perf_counter() - t0
        print(f"{L:6.1f} {N:5d} {grid.h:9.5f} {pt.energy:+15.8f} {pt.n_iters:7d} {str(pt.converged):>6} "
              f"{dt:7.2f}s", flush=True)
        rows.append({"L": L, "N": N, "h": grid.h, "E": pt.energy, "iters": pt.n_iters,
                     "converged": pt.converged, "seconds": dt})
    print()
    ok = [r for r in rows if r["converged"]]
    hs = [r["h"] for r in ok]
    drift = bool(hs) and (max(hs) - min(hs)) > 1e-4
    if drift:
        print(f"  WARNING: h drifted over {min(hs):.5f}..{max(hs):.5f}; box and resolution errors are "
              f"confounded and the fit is unreliable. Use a target_h that divides every L.")
        groups: dict = {}
        for r in ok:
            groups.setdefault(round(r["h"], 10), []).append(r)
        for h, grp in sorted(groups.items()):
            if len(grp) >= 2:
                es = [r["E"] for r in grp]
                which = ", ".join("L=%g" % r["L"] for r in grp)
                print(f"  controlled at h = {h:.5f} ({which}): spread {1e3 * (max(es) - min(es)):.2f} mHa")
    fit = _report("E(L -> inf)", [1.0 / r["L"] for r in ok], [r["E"] for r in ok], "Ha") if len(ok) >= 3 else None
    return {"rows": rows, "fit": fit, "h_drift": drift}


def sweep_geometry(case, Ns, L, order, geom_steps, lr, scf_iters, precision="fp64"):
    """Relaxed geometry against h."""
    print(f"{case.name}: relaxed geometry vs grid spacing at fixed L = {L} a0, {precision}")
    print(f"{'N':>5} {'h (a0)':>9} {'R (a0)':>10} {'angle':>9} {'E (Ha)':>15} {'conv':>6} {'time':>8}")
    rows = []
    for N in Ns:
        grid = Grid3D(N=N, L=L)
        t0 = time.perf_counter()
        out = case.optimize(grid, geom_steps=geom_steps, learning_rate=lr, scf_max_iters=scf_iters, order=order,
                            precision=precision)
        dt = time.perf_counter() - t0
        print(f"{N:5d} {grid.h:9.5f} {out['R']:10.5f} {out['angle']:9.3f} {out['E']:+15.8f} "
              f"{str(out['converged']):>6} {dt:7.2f}s", flush=True)
        rows.append(dict(out, N=N, h=grid.h, seconds=dt))
    print()
    ok = [r for r in rows if r["converged"]]
    hs = [r["h"] for r in ok]
    fits = {"R": _report("R(h -> 0)", hs, [r["R"] for r in ok], "a0")}
    if ok and not math.isnan(ok[0]["angle"]):
        fits["angle"] = _report("angle(h -> 0)", hs, [r["angle"] for r in ok], "deg")
    fits["E"] = _report("E(h -> 0)", hs, [r["E"] for r in ok], "Ha")
    return {"rows": rows, "fit": fits}


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--molecule", choices=sorted(CASES), default="water")
    ap.add_argument("--mode", choices=["energy", "box", "geometry"], default="energy")
    ap.add_argument("--N", type=int, nargs="+", default=None, help="grid sizes (energy / geometry modes)")
    ap.add_argument("--L", type=float, default=None, help="box side (energy / geometry modes)")
    ap.add_argument("--box-L", type=float, nargs="+", default=[12.0, 14.0, 16.0, 18.0])
    ap.add_argument("--target-h", type=float, default=0.175, help="spacing held in box mode")
    ap.add_argument("--order", type=int, choices=[2, 4], default=4)
    ap.add_argument("--scf-iters", type=int, default=80)
    ap.add_argument("--geom-steps", type=int, default=30)
    ap.add_argument("--lr", type=float, default=0.05)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--json", default=None, help="also write the rows and fits to this file")
    args = ap.parse_args(argv)
    case = CASES[args.molecule]()
    L = args.L if args.L is not None else case.default_L
    if args.mode == "energy":
        out = sweep_energy(case, args.N or [32, 48, 64, 80, 96, 112, 128], L, args.order, args.scf_iters,
                           args.precision)
    elif args.mode == "box":
        out = sweep_box(case, args.box_L, args.target_h, args.order, args.scf_iters, args.precision)
    else:
        out = sweep_geometry(case, args.N or [32, 48, 64, 80, 96], L, args.order, args.geom_steps, args.lr,
                             args.scf_iters, args.precision)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(out, f, indent=1)
    return out


if __name__ == "__main__":
    main()
