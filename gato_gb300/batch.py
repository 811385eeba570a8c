"""Many independent molecules on one GPU: the batched mixed-size workload.

A batch is a list of closed-shell systems (H2, LiH, HCl, H2O) of different
grid sizes and spacings. One system's SCF on a 64^3 or 96^3 grid keeps only
part of a GB300 busy (its FFT passes work on 128^3 or 192^3 doubled grids
and its launches are short), so ``solve_batch`` runs the systems
concurrently: a pool of worker threads, each on its own CUDA stream with its
own Poisson plans and non-local operators (the caches are per thread), each
taking the next system from a shared queue, largest first. The library
calls release the GIL, so the workers submit launches in parallel. Every
system gets its SCF energy and its Hellmann-Feynman forces.

``draw_systems`` builds the seeded 48-system workload: species drawn from
{H2 (d 1.2-1.6 bohr, softened Coulomb), LiH (d 2.8-3.2), HCl (d 2.2-2.6),
H2O (R_OH = 1.81, 104.5 deg, +-0.05 bohr jitter)}, grids of 64, 96, 128 or
160 points per axis and h uniform in [0.2, 0.3] bohr.
"""
from __future__ import annotations

import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .geometry import Nuclei, diatomic_along_z
from .grid import Grid3D
from .physics import _molecule as mol
from .physics.water import water_initial_geometry
from .pseudopotentials import lookup

SPECIES = ("H2", "LiH", "HCl", "H2O")
GRIDS = (64, 96, 128, 160)


@dataclass
class SystemSpec:
    name: str
    nuclei: Nuclei
    N: int
    h: float
    elements: tuple | None = None     # HGH parameters; None: softened Coulomb nuclei (H2)

    @property
    def grid(self) -> Grid3D:
        return Grid3D(self.N, self.N * self.h)

    def model(self):
        return mol.HGHModel(self.elements) if self.elements is not None else mol.SoftCoulombModel(None)

    def n_occ(self) -> int:
        return self.model().n_electrons(self.nuclei) // 2


@dataclass
class SystemResult:
    spec: SystemSpec
    point: mol.MoleculePoint
    forces: torch.Tensor            # (K, 3), Ha / bohr
    seconds: float
    stream: int
    extra: dict = field(default_factory=dict)


def draw_systems(n: int = 48, seed: int = 0, grids=GRIDS) -> list[SystemSpec]:
    """The seeded mixed-size workload (species, grid, spacing and geometry per system)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = SPECIES[int(rng.integers(len(SPECIES)))]
        N = int(grids[int(rng.integers(len(grids)))])
        h = float(rng.uniform(0.2, 0.3))
        if kind == "H2":
            nuc, el = diatomic_along_z(float(rng.uniform(1.2, 1.6)), Z1=1.0), None
        elif kind == "LiH":
            nuc, el = diatomic_along_z(float(rng.uniform(2.8, 3.2)), Z1=3.0, Z2=1.0), (lookup("Li"), lookup("H"))
        elif kind == "HCl":
            nuc, el = diatomic_along_z(float(rng.uniform(2.2, 2.6)), Z1=1.0, Z2=17.0), (lookup("H"), lookup("Cl"))
        else:
            w = water_initial_geometry(1.81, 104.5)
            nuc = Nuclei(w.positions + torch.tensor(rng.uniform(-0.05, 0.05, (3, 3))), w.charges)
            el = (lookup("O"), lookup("H"), lookup("H"))
        out.append(SystemSpec(f"{kind}#{i}", nuc, N, h, el))
    return out


def solve_system(spec: SystemSpec, *, precision: str = "mixed", max_iters: int = 60, tol: float = 1e-6,
                 mixing: float = 0.5, order: int = 4, initial_orbitals=None) -> tuple:
    """SCF at the spec's geometry plus the Hellmann-Feynman forces, on the current stream."""
    model, grid = spec.model(), spec.grid
    n_occ = 1 if spec.elements is None else None
    p = mol.solve_closed_shell(model, spec.nuclei, grid, n_occ=n_occ, max_iters=max_iters, tol=tol,
                               mixing=mixing, order=order, lanczos_iters=None, initial_orbitals=initial_orbitals,
                               precision=precision)
    F = -mol.bo_grad_model(model, p.nuclei.positions, p.nuclei.charges, p.orbitals, grid, order)
    return p, F


def solve_batch(specs, *, precision: str = "mixed", streams: int = 8, max_iters: int = 60, tol: float = 1e-6,
                mixing: float = 0.5, order: int = 4) -> tuple[list[SystemResult], float]:
    """Solve every system; returns (results in input order, wall seconds).

    ``streams`` worker threads each own a CUDA stream; systems are handed out
    largest grid first so the big ones do not trail at the end.
    """
    dev = torch.device("cuda", torch.cuda.current_device())
    order_idx = sorted(range(len(specs)), key=lambda i: -specs[i].N ** 3 * max(1, specs[i].n_occ()))
    work: queue.Queue = queue.Queue()
    for i in order_idx:
        work.put(i)
    results: list = [None] * len(specs)
    errors: list = []
    seq = [0] * max(1, streams)   # position of each system in its worker's sequence

    def worker(k: int):
        torch.cuda.set_device(dev)
        s = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(s):
            while not errors:
                try:
                    i = work.get_nowait()
                except queue.Empty:
                    return
                t0 = time.perf_counter()
                try:
                    p, F = solve_system(specs[i], precision=precision, max_iters=max_iters, tol=tol,
                                        mixing=mixing, order=order)
                    s.synchronize()
                except BaseException as e:   # surfaced to the caller after the pool stops
                    errors.append(e)
                    return
                results[i] = SystemResult(specs[i], p, F, time.perf_counter() - t0, k,
                                          {"worker_seq": seq[k]})
                seq[k] += 1

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    threads = [threading.Thread(target=worker, args=(k,), daemon=True) for k in range(max(1, streams))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if errors:
        raise errors[0]
    return results, wall


def summarize(results, wall: float) -> dict:
    """Throughput and per-system figures of a finished batch."""
    iters = sum(r.point.n_iters for r in results)
    return {"systems": len(results), "wall_s": wall, "systems_per_s": len(results) / wall,
            "scf_iterations": iters, "scf_iterations_per_s": iters / wall,
            "converged": sum(bool(r.point.converged) for r in results),
            "per_system": [{"name": r.spec.name, "N": r.spec.N, "h": round(r.spec.h, 5), "E": r.point.energy,
                            "iters": r.point.n_iters, "max_abs_F": float(r.forces.abs().max()),
                            "s": round(r.seconds, 3)} for r in results]}


def fp64_check(result: SystemResult, *, fp64_iters: int = 30, tol: float = 1e-9, order: int = 4,
               mixing: float = 0.5) -> dict:
    """Mixed against FP64 for one solved system.

    Energy: an FP64 SCF continued from the mixed orbitals to ``tol``; |dE| is
    meaningful when the mixed SCF itself was converged tightly. Forces: the
    FP64 force evaluation on the same (mixed) orbitals against the mixed
    one, i.e. the precision of the force path alone (forces are first order
    in any SCF stopping error, so comparing two separately stopped SCFs
    would measure the stopping, not the arithmetic).
    """
    spec, model, grid = result.spec, result.spec.model(), result.spec.grid
    orb64 = result.point.orbitals.to(torch.float64)
    p = result.point
    F64 = -mol.bo_grad_model(model, p.nuclei.positions, p.nuclei.charges, orb64, grid, order)
    n_occ = 1 if spec.elements is None else None
    p64 = mol.solve_closed_shell(model, spec.nuclei, grid, n_occ=n_occ, max_iters=fp64_iters, tol=tol,
                                 mixing=mixing, order=order, lanczos_iters=None, initial_orbitals=orb64,
                                 precision="fp64")
    return {"name": spec.name, "N": spec.N, "abs_dE": abs(p64.energy - p.energy),
            "max_abs_dF": float((F64 - result.forces).abs().max()), "fp64_iters": p64.n_iters,
            "fp64_converged": bool(p64.converged), "mixed_converged": bool(p.converged),
            "finite": bool(math.isfinite(p64.energy))}
