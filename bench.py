#!/usr/bin/env python
"""H2O 128^3 RHF Fock-applies/s and force time, mixed precision vs plain FP64.

Workload (one step = one block Fock apply): water with HGH pseudopotentials
(O Z_ion=6, H Z_ion=1) at R_OH = 1.81 bohr, 104.5 deg plus seeded +-0.05 bohr
jitter, on a 128^3 grid with h = 0.25 bohr and the 13-point Laplacian; four
seeded orthonormal occupied orbitals; F phi_i for all four orbitals with the
10 pair Poisson solves J[phi_i phi_j] on the 256^3 doubled grid. `value` is
the mixed path (FP32 fields/stencil/FFT/exchange, FP64 and float-float
reductions) with inputs resident in HBM; `e2e` is the same through the public
API with the orbitals copied in from pinned host memory and the result copied
back every step. Also reported: the plain FP64 rate, matvec (one vector,
4 pair solves) rates, |Delta E| of the energy terms mixed vs FP64, the force
time of both paths, the roofline of the dominant kernel and of the stencil,
and the CPU baseline (the NumPy restatement of the reference on the host).

Launch: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
(N > 1 via torch.distributed.run: independent replicas, one per GPU).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT, H_DEFAULT, N_OCC = 128, 0.25, 4
# DRAM read + write of one x-pass launch (5 fields, 128^3) in the one-kernel ncu capture summarised
# in profiles/x_pass_fmi_h2o128_f32_packed.md (a recorded figure, not measured by this run)
FMI_TRAFFIC_128 = 366_514_944 + 274_889_216
FMI_TRAFFIC_SOURCE = "profiles/x_pass_fmi_h2o128_f32_packed.md (ncu, same kernel and workload; not re-measured here)"
FMI_LIMITER = ("latency: packed two-line FFT, 3 CTAs (12 warps) per SM by shared memory; issue 43%, FMA pipe 58%, "
               "shared-memory wavefronts 62% (ncu); a 4-CTA layout measured no faster")
METRIC = "H2O 128^3 RHF block Fock-applies/s (mixed FP32/FP64 at |dE|<1uHa) and force time"
UNIT = "Fock-applies/s"


def workload_name(N: int, h: float) -> str:
    """The bench workload, named the same on both arms."""
    return (f"H2O HGH {N}^3 h={h} block Fock apply: 4 orbitals, 10 pair Poisson solves "
            f"on the {2 * N}^3 doubled grid")


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def synthetic_orbitals(centres, N: int, h: float, n_occ: int, rng):
    """n_occ orthonormal smooth orbitals (float64, host numpy) on the N^3 grid of spacing h: Gaussians
    of seeded width around the given centres (cycled) times a seeded linear factor, orthonormalised by
    Gram-Schmidt in the grid inner product."""
    import numpy as np
    L = N * h
    a = -L / 2 + (np.arange(N) + 0.5) * h
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    orbs = np.empty((n_occ, N, N, N))
    for k in range(n_occ):
        c = centres[k % len(centres)] + rng.uniform(-0.3, 0.3, 3)
        al = rng.uniform(0.4, 0.9)
        w = rng.uniform(-0.3, 0.3, 3)
        orbs[k] = np.exp(-al * ((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2)) * (
            1.0 + w[0] * X + w[1] * Y + w[2] * Z)
    dV = h ** 3
    for i in range(n_occ):
        for j in range(i):
            orbs[i] -= np.sum(orbs[i] * orbs[j]) * dV * orbs[j]
        orbs[i] /= math.sqrt(np.sum(orbs[i] ** 2) * dV)
    return orbs


def synthetic_water(N: int, h: float, seed: int = 2024):
    """Seeded geometry and four orthonormal smooth orbitals (float64, host numpy)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    half = math.radians(104.5) / 2
    pos = np.array([[0.0, 0.0, 0.0], [1.81 * math.sin(half), 0.0, 1.81 * math.cos(half)],
                    [-1.81 * math.sin(half), 0.0, 1.81 * math.cos(half)]])
    pos = pos + rng.uniform(-0.05, 0.05, (3, 3))
    return pos, synthetic_orbitals(pos, N, h, N_OCC, rng)


def identical_orbital_energies(nuclei, elements, grid, orbs):
    """Total energy of the same orbitals three ways (Ha): the FP64 path; the mixed path as it reports
    energies (FP64 terms of the FP32-rounded orbitals); and the FP32 operator's own energy terms, which
    a mixed SCF uses only while the energy still moves by more than ~1e-4 Ha per iteration."""
    import torch
    from gato_gb300.pseudopotentials import hgh_local_potential, nonlocal_for
    from gato_gb300.scf import decompose_rhf_energy, from_fields
    f64 = torch.tensor(orbs, device="cuda", dtype=torch.float64).contiguous()
    f32 = f64.to(torch.float32).contiguous()
    out = {}
    for name, fields, dt in (("fp64", f64, torch.float64), ("mixed", f32.to(torch.float64), torch.float64),
                             ("fp32_operator", f32, torch.float32)):
        V = hgh_local_potential(nuclei, elements, grid, dt)
        nl = nonlocal_for(nuclei, elements, grid, dt)
        t = decompose_rhf_energy(from_fields(fields), V, grid, order=4, V_nl_apply=nl)
        out[name] = float(t.total)
    return {"E_fp64": out["fp64"], "E_mixed": out["mixed"], "E_fp32_operator": out["fp32_operator"],
            "abs_dE_mixed_Ha": abs(out["mixed"] - out["fp64"]),
            "abs_dE_fp32_operator_Ha": abs(out["fp32_operator"] - out["fp64"])}


def energy_gate_160():
    """The 1e-6 Ha gate at 160^3: HCl#17 of the seeded 48-system draw (h = 0.2015 bohr, HGH H and Cl)
    with four seeded orthonormal orbitals, energies of identical orbitals as in the headline."""
    import numpy as np
    from gato_gb300.batch import draw_systems
    spec = [s for s in draw_systems(48, seed=0) if s.name == "HCl#17"][0]
    orbs = synthetic_orbitals(spec.nuclei.positions.numpy(), spec.N, spec.h, 4, np.random.default_rng(17))
    r = identical_orbital_energies(spec.nuclei, spec.elements, spec.grid, orbs)
    return dict(r, system=f"{spec.name} N={spec.N} h={spec.h:.4f}")


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 50 ms during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.path = gpu, None, f"/tmp/gato_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        # the region starts once sampling has (nvidia-smi takes a moment to start)
        t0 = time.time()
        while self.proc is not None and time.time() - t0 < 3.0:
            if os.path.exists(self.path) and os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.remove(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def job_rate(t_local: float, steps: int, world: int, dist=None, device=None):
    """Whole-job rate of `world` replicas that each ran `steps` steps, the local one in `t_local`
    seconds: the job took the slowest rank's time (an all-reduce MAX when world > 1), and every
    rank's steps count. Returns (rate, job seconds)."""
    t_max = t_local
    if world > 1:
        import torch
        tt = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt)
    return world * steps / t_max, t_max


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_block_apply_rate(pos, orbs, N, h):
    """The NumPy restatement of the reference (oracle) on the host cores."""
    import numpy as np
    from oracle import gato_np as o
    g = o.Grid3D(N, N * h)
    nuc = o.Nuclei(pos, np.array([8.0, 1.0, 1.0]))
    el = o.water_hgh_elements()
    V = o.hgh_local_potential(nuc, el, g) + o.hartree_potential(o._density(np.moveaxis(orbs, 0, -1)), g)
    nl = lambda p: o.hgh_nonlocal_apply(p, nuc, el, g)  # noqa: E731
    o.fock_apply_block(orbs[:1], V, g, order=4, nl=nl)   # warm the kernel-spectrum cache
    t0 = time.perf_counter()
    o.fock_apply_block(orbs, V, g, order=4, nl=nl)
    dt = time.perf_counter() - t0
    return 1.0 / dt, dt


def run_reference(args):
    """`--impl reference`: the reference algorithm's CPU implementation (the
    oracle port; the JAX reference is not installable offline), same metric."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from oracle import gato_np as o
    N, h = args.N, H_DEFAULT
    pos, orbs = synthetic_water(N, h)
    g = o.Grid3D(N, N * h)
    nuc = o.Nuclei(pos, np.array([8.0, 1.0, 1.0]))
    el = o.water_hgh_elements()
    V = o.hgh_local_potential(nuc, el, g) + o.hartree_potential(o._density(np.moveaxis(orbs, 0, -1)), g)
    nl = lambda p: o.hgh_nonlocal_apply(p, nuc, el, g)  # noqa: E731
    for _ in range(args.warmup):
        o.fock_apply_block(orbs, V, g, order=4, nl=nl)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.fock_apply_block(orbs, V, g, order=4, nl=nl)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water geometry and orbitals)",
            "config": {"workload": workload_name(N, h), "precision": "fp64", "N": N, "h": h, "n_occ": N_OCC,
                       "parallelism": "rank 0 only (host cores)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} block Fock applies of the {N}^3 workload"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def e2e_pipelined(st, st_b, host_in, steps):
    """Seconds for `steps` block applies through the public API from pinned host memory, pipelined.

    Two operators (each with its own orbital buffer, Poisson plan and projector scratch) alternate,
    each computing on its own stream: step k's host-to-device copy runs on an upload stream, step k's
    result comes back on a download stream, and step k's kernels may overlap step k-1's. Each step
    still copies its own inputs in and its whole result out; the window runs from the first upload
    to the last download."""
    import torch
    comp = torch.cuda.current_stream()
    comps = [comp, torch.cuda.Stream()]
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    ops, bufs, outs = [st["op"], st_b["op"]], [st["fields"], st_b["fields"]], [st["out"], st_b["out"]]
    hosts = [torch.empty_like(host_in).pin_memory() for _ in range(2)]
    ev = lambda: torch.cuda.Event()   # noqa: E731
    try:   # each operator's block apply as a graph replay, as in the headline
        graphs = [op.block_graph(o) for op, o in zip(ops, outs)]
        steps_fn = [g.replay for g in graphs]
    except Exception:
        steps_fn = [lambda b=b: ops[b].apply_block(outs[b]) for b in range(2)]

    def run(n):
        done = [None, None]   # compute of the buffer's previous step (frees its input and output)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(comp)
        up.wait_event(t0)
        comps[1].wait_event(t0)
        loaded = []
        for k in range(n):
            b = k % 2
            cs = comps[b]
            with torch.cuda.stream(up):
                if done[b] is not None:
                    up.wait_event(done[b])
                bufs[b].copy_(host_in, non_blocking=True)
                e = ev()
                e.record(up)
                loaded.append(e)
            cs.wait_event(loaded[k])
            if k >= 2:
                cs.wait_event(dl[b])   # the buffer's previous result is home
            with torch.cuda.stream(cs):
                steps_fn[b]()
            done[b] = ev()
            done[b].record(cs)
            with torch.cuda.stream(down):
                down.wait_event(done[b])
                hosts[b].copy_(outs[b], non_blocking=True)
                dl[b] = ev()
                dl[b].record(down)
        comp.wait_stream(comps[1])
        comp.wait_stream(down)
        t1.record(comp)
        t1.synchronize()
        return t0.elapsed_time(t1) * 1e-3

    dl = [None, None]
    run(4)
    torch.cuda.synchronize()
    return run(steps)


def cufft_comparator(st, N, h, eps, timed, steps):
    """The reference's Hockney solve (solvers/poisson.py:47-57) on cuFFT through torch.fft, timed beside
    this library's pipeline on the same FP32 inputs. Comparator only: J = irfftn(rfftn(pad(rho)) *
    rfftn(G))[:N, :N, :N] dV with rfftn(G) built once (the reference rebuilds it on every call).
    Reported: one Hartree solve both ways, and the 10 pair potentials J[phi_a phi_b] of a block apply
    on cuFFT against this library's whole block apply (which also runs the stencil, the non-local part
    and the exchange accumulation)."""
    import torch
    from gato_gb300.solvers.poisson import hartree_potential
    from gato_gb300.grid import Grid3D
    dev = st["fields"].device
    M = 2 * N
    idx = torch.arange(M, device=dev, dtype=torch.float64)
    disp = torch.where(idx < N, idx * h, (idx - M) * h)
    G = 1.0 / torch.sqrt(disp[:, None, None] ** 2 + disp[None, :, None] ** 2 + disp[None, None, :] ** 2 + eps * eps)
    ghat = torch.fft.rfftn(G.to(torch.float32)) * (h ** 3)
    del G
    phi = st["fields"]
    n = phi.shape[0]
    pairs = [(a, b) for a in range(n) for b in range(a, n)]
    pad = torch.zeros((len(pairs), M, M, M), dtype=torch.float32, device=dev)

    def pair_solves():
        for i, (a, b) in enumerate(pairs):
            pad[i, :N, :N, :N] = phi[a] * phi[b]
        J = torch.fft.irfftn(torch.fft.rfftn(pad, dim=(1, 2, 3)) * ghat, s=(M, M, M), dim=(1, 2, 3))
        return J[:, :N, :N, :N].contiguous()

    rho = (2.0 * (phi * phi).sum(0)).contiguous()
    pad1 = torch.zeros((M, M, M), dtype=torch.float32, device=dev)

    def hartree_cufft():
        pad1[:N, :N, :N] = rho
        return torch.fft.irfftn(torch.fft.rfftn(pad1) * ghat, s=(M, M, M))[:N, :N, :N].contiguous()

    g = Grid3D(N, N * h)
    t_pairs = timed(pair_solves, steps, 2)
    t_hc = timed(hartree_cufft, steps, 2)
    t_hg = timed(lambda: hartree_potential(rho, g, eps), steps, 2)
    err = float(torch.max(torch.abs(hartree_cufft() - hartree_potential(rho, g, eps))) /
                torch.max(torch.abs(hartree_cufft())))
    out = {"hartree_us": {"gato": 1e6 * sum(t_hg) / len(t_hg), "cufft": 1e6 * sum(t_hc) / len(t_hc),
                          "max_rel_diff": err},
           "pair_potentials_10_us_cufft": 1e6 * sum(t_pairs) / len(t_pairs),
           "note": "torch.fft (cuFFT) FP32 rfftn/irfftn of the zero-padded 2N^3 grid with a precomputed "
                   "kernel spectrum; comparator only, never on the product path"}
    del pad, pad1, ghat
    torch.cuda.empty_cache()
    return out


def run_gato(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from gato_gb300 import _lib
    from gato_gb300.geometry import Nuclei
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import bo_grad_positions, water_hgh_elements
    from gato_gb300.pseudopotentials import hgh_local_potential, nonlocal_for
    from gato_gb300.scf import Operator, _density_fields, from_fields, pair_fields
    from gato_gb300.solvers.poisson import get_plan

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    N, h = args.N, H_DEFAULT
    g = Grid3D(N, N * h)
    dev = torch.device("cuda", local)
    pos, orbs = synthetic_water(N, h)
    nuc = Nuclei(torch.tensor(pos), torch.tensor([8.0, 1.0, 1.0], dtype=torch.float64))
    el = water_hgh_elements()
    n3 = N ** 3
    eps = h / 2

    def build(dtype):
        fields = torch.tensor(orbs, device=dev).to(dtype).contiguous()
        V_loc = hgh_local_potential(nuc, el, g, dtype)
        nl = nonlocal_for(nuc, el, g, dtype)
        plan = get_plan(N, h, eps, dtype, pair_fields(N_OCC))
        V_tot = (V_loc + plan.potential(_density_fields(fields))).contiguous()
        op = Operator(g, dtype, 4, "dirichlet")
        op.set_potential(V_tot)
        op.set_nonlocal(nl)
        op.set_exchange(plan, fields)
        return dict(fields=fields, V_loc=V_loc, nl=nl, plan=plan, op=op, out=torch.empty_like(fields))

    s32, s64 = build(torch.float32), build(torch.float64)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    from gato_gb300.autotune import tune_plan
    tuned = {}
    from gato_gb300.autotune import tune_block_epilogue
    for name, st in (("mixed", s32), ("fp64", s64)):
        step = lambda st=st: st["op"].apply_block(st["out"])  # noqa: E731
        best = tune_plan(st["plan"], step, key="block", engines=(0, 2))
        epi = tune_block_epilogue(st["op"], step, key="block")
        tuned[name] = {"group": best["group"], "engine": best["engine"],
                       "candidates_ms": {f'{c["engine"]}:{c["group"]}': round(c["ms"], 4)
                                         for c in best["candidates"]},
                       "block_epilogue": epi["epilogue"],
                       "epilogue_ms": {str(c["epilogue"]): round(c["ms"], 4) for c in epi["candidates"]}}

    # a second FP32 operator over its own orbital buffer, Poisson plan and projector scratch, so that
    # two block applies can be in flight on two streams (the plan's spectral buffers and the
    # projectors' overlap sums are per object, so one object serves one stream at a time)
    from gato_gb300.autotune import set_plan
    from gato_gb300.solvers.poisson import PoissonPlan
    plan_b = PoissonPlan(N, h, eps, torch.float32, pair_fields(N_OCC))
    set_plan(plan_b, tuned["mixed"]["group"], tuned["mixed"]["engine"])
    op_b = Operator(g, torch.float32, 4, "dirichlet")
    op_b.set_potential(s32["op"]._keep["V"])
    op_b.set_nonlocal(nonlocal_for(nuc, el, g, torch.float32))
    op_b.tune(s32["op"].block_epilogue)
    fields_b = s32["fields"].clone()
    op_b.set_exchange(plan_b, fields_b)
    s32b = dict(op=op_b, fields=fields_b, out=torch.empty_like(s32["out"]))

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        evs = []
        for _ in range(steps):
            flush.fill_(1.0)                     # L2 flush, outside the timed events
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            evs.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) * 1e-3 for a, b in evs]

    # ---- headline: mixed block Fock apply, inputs resident ----------------------
    op32 = s32["op"]
    for _ in range(args.warmup):
        op32.apply_block(s32["out"])
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    # the step as direct launches, then as a replay of the same launches captured once in a CUDA graph;
    # clocks are sampled over both, bracketed by 0.5 s of the same step before and after (untimed):
    # the timed region alone is ~10 ms, shorter than the sampling interval
    def load_pad(fn, seconds=0.5):
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            for _ in range(20):
                fn()
            torch.cuda.synchronize()

    clk = ClockSampler(local).__enter__()
    load_pad(lambda: op32.apply_block(s32["out"]))
    direct = timed(lambda: op32.apply_block(s32["out"]), args.steps, 0)
    graph = None
    try:
        l0 = _lib.launch_count()
        graph = op32.block_graph(s32["out"])
        per_step = (_lib.launch_count() - l0) // 2      # one warm-up run and the captured run
    except Exception as exc:   # capture refused: the direct launches are the step
        graph_error = f"{type(exc).__name__}: {exc}"
        per_step = None
    l0 = _lib.launch_count()
    try:
        if graph is not None:
            times = timed(graph.replay, args.steps, 3)
            launches = per_step * args.steps
        else:
            times = timed(lambda: op32.apply_block(s32["out"]), args.steps, 0)
            launches = (_lib.launch_count() - l0) // max(args.steps, 1) * args.steps
        torch.cuda.synchronize()
        load_pad(graph.replay if graph is not None else (lambda: op32.apply_block(s32["out"])))
    finally:
        clk.__exit__(None, None, None)
    value, t_max = job_rate(sum(times), args.steps, world, dist, dev)

    # two steps in flight: the second operator's step replays on its own stream beside the first's
    # (no L2 flush between steps here: each step streams ~2.4 GB, far more than L2 holds)
    two_streams = None
    if graph is not None:
        graph_b = s32b["op"].block_graph(s32b["out"])
        sb = torch.cuda.Stream()

        def two(n):
            cur = torch.cuda.current_stream()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(cur)
            sb.wait_stream(cur)
            for _ in range(n // 2):
                graph.replay()
                with torch.cuda.stream(sb):
                    graph_b.replay()
            cur.wait_stream(sb)
            e1.record(cur)
            e1.synchronize()
            return e0.elapsed_time(e1) * 1e-3
        two(6)
        n2 = 2 * max(3, args.steps // 2)
        two_streams = {"value": n2 / two(n2), "steps": n2,
                       "mode": "two operators, each step a graph replay on its own stream"}
        del graph_b

    # ---- plain FP64 and matvec rates ----------------------------------------------
    k64 = max(2, args.steps // 4)
    t64 = timed(lambda: s64["op"].apply_block(s64["out"]), k64, 1)
    rate64 = k64 / sum(t64)
    psi32, psi64 = s32["fields"][1].clone(), s64["fields"][1].clone()
    o32, o64 = torch.empty_like(psi32), torch.empty_like(psi64)
    tm32 = timed(lambda: op32.apply(psi32, o32), args.steps, 2)
    tm64 = timed(lambda: s64["op"].apply(psi64, o64), k64, 1)

    # ---- accuracy: energies of the same orbitals, mixed vs FP64 --------------------
    e32 = s32["op"].energy_terms(s32["V_loc"]).cpu().numpy()
    e64 = s64["op"].energy_terms(s64["V_loc"]).cpu().numpy()
    gate128 = identical_orbital_energies(nuc, el, g, orbs)

    # ---- force time ---------------------------------------------------------------
    def force_ms(st):
        o = from_fields(st["fields"])
        bo_grad_positions(nuc.positions, nuc.charges, o, el, g)   # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f = bo_grad_positions(nuc.positions, nuc.charges, o, el, g)
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0), f
    f32_ms, F32 = force_ms(s32)
    f64_ms, F64 = force_ms(s64)
    dF = float(torch.max(torch.abs(F32 - F64)))

    # ---- roofline: dominant kernel (x-pass: FFT, kernel multiply, inverse FFT) ----
    peak, peak_kind = measured_peaks()
    M, Hh = 2 * N, N + 1
    nf = (N_OCC * (N_OCC + 1) // 2 + 1) // 2
    plan = s32["plan"]
    tx = timed(lambda: _lib.call("gato_poisson_stage", plan.handle, 2, nf, torch.cuda.current_stream().cuda_stream),
               max(3, args.steps), 2)
    tx_avg = sum(tx) / len(tx)
    bytes_x = nf * (2 * N * M * M * 8) + Hh ** 3 * 4
    # stencil: 3 N^3 s per field (psi, V, out), four fields per launch
    from gato_gb300.operators import stencil
    st_in, st_out = s32["fields"], torch.empty_like(s32["fields"])
    V32 = s32["op"]._keep["V"]
    from gato_gb300.autotune import tune_stencil
    st_step = lambda: stencil(st_in, h, "dirichlet", 4, -0.5 / h ** 2, V=V32, out=st_out)  # noqa: E731
    st_best = tune_stencil(st_step, key="bench")
    ts = timed(st_step, max(3, args.steps), 2)
    ts_single = sum(ts) / len(ts)      # one launch after an L2 flush, event latency included
    # steady state: K launches back to back over 4 rotating input/output sets (302 MB, more than
    # L2 holds), one event pair around them, the average launch duration
    sets = [(st_in.clone(), V32.clone(), torch.empty_like(st_out)) for _ in range(4)]
    K = 4 * max(2, args.steps // 4)
    for a_, v_, o_ in sets:
        stencil(a_, h, "dirichlet", 4, -0.5 / h ** 2, V=v_, out=o_)
    flush.fill_(1.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(K):
        a_, v_, o_ = sets[k % 4]
        stencil(a_, h, "dirichlet", 4, -0.5 / h ** 2, V=v_, out=o_)
    e1.record()
    e1.synchronize()
    ts_avg = e0.elapsed_time(e1) * 1e-3 / K
    del sets
    bytes_s = 3 * n3 * 4 * N_OCC

    # ---- cuFFT comparator ----------------------------------------------------------
    cufft = cufft_comparator(s32, N, h, eps, timed, max(3, args.steps))

    # ---- e2e: public API with host buffers ---------------------------------------
    host_in = torch.tensor(orbs, dtype=torch.float32).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()

    def e2e_step():
        s32["fields"].copy_(host_in, non_blocking=True)
        op32.apply_block(s32["out"])
        host_out.copy_(s32["out"], non_blocking=True)
    te = timed(e2e_step, args.steps, 2)
    e2e_serial = world * args.steps / sum(te)
    e2e_val, _ = job_rate(e2e_pipelined(s32, s32b, host_in, args.steps), args.steps, world, dist, dev)

    # ---- the energy gate at 160^3 (after every timing: its FP64 plans are large) ------
    gate160 = energy_gate_160() if rank == 0 else None

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu:
        rate, dt = cpu_block_apply_rate(pos, orbs, N, h)
        cpu = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"1 block Fock apply of the {N}^3 workload ({dt:.2f} s) with scipy.fft on all cores"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded water geometry and orbitals)",
        "config": {"workload": workload_name(N, h), "precision": "mixed", "N": N, "h": h,
                   "n_occ": N_OCC, "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas",
                   "autotune": tuned},
        "clocks": dict(clk.summary(), window="the timed direct and graph steps, bracketed by 0.5 s of the same "
                                              "step before and after"),
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": host_in.numel() * 4,
                "d2h_bytes_per_step": host_out.numel() * 4,
                "mode": "two-deep pipeline: step k+1's orbitals copy in and step k-1's result copies out "
                        "on their own streams while step k computes; consecutive steps alternate between "
                        "two operators (own plan and projector scratch) computing on two streams, so "
                        "their kernels may overlap; every step copies its own inputs and result (no L2 "
                        "flush: the step streams ~2.4 GB of spectral buffers)",
                "serial_value": e2e_serial},
        "gpu_launches": int(launches),
        "cuda_graph": ({"used": True, "kernels_per_step": per_step,
                        "direct_launch_value": world * args.steps / sum(direct),
                        "two_streams": two_streams} if graph is not None
                       else {"used": False, "error": graph_error,
                             "direct_launch_value": world * args.steps / sum(direct)}),
        "roofline": {"kernel": "packed::k_colsp<16,16,8,FMI> (x FFT, kernel multiply, inverse x FFT; "
                               "two lines per thread in f32x2)", "bound": "hbm",
                     "achieved": bytes_x / tx_avg / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": bytes_x / tx_avg / 1e9 / peak,
                     "traffic": FMI_TRAFFIC_128 if N == 128 else None,
                     "traffic_source": FMI_TRAFFIC_SOURCE if N == 128 else None, "peak_kind": peak_kind,
                     "algorithmic_bytes": bytes_x, "avg_launch_us": tx_avg * 1e6,
                     "limiter": FMI_LIMITER},
        "roofline_stencil": {"bound": "hbm", "achieved": bytes_s / ts_avg / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": bytes_s / ts_avg / 1e9 / peak, "avg_launch_us": ts_avg * 1e6,
                             "timing": "average of back-to-back launches over 4 rotating input sets (302 MB)",
                             "single_launch_after_flush": {"us": ts_single * 1e6,
                                                           "frac": bytes_s / ts_single / 1e9 / peak},
                             "rows_per_thread": st_best["rows"],
                             "candidates_ms": {str(c["rows"]): round(c["ms"], 5) for c in st_best["candidates"]}},
        "cpu_baseline": cpu,
        "cufft_comparator": dict(cufft, gato_block_apply_us=1e6 * t_max / args.steps),
        "fp64_block_applies_per_s": rate64,
        "speedup_mixed_vs_fp64": value / world / rate64,
        "matvec_applies_per_s": {"mixed": args.steps / sum(tm32), "fp64": k64 / sum(tm64)},
        "energy_terms": {"fp32_operator": e32.tolist(), "fp64": e64.tolist(),
                         "order": ["kinetic", "v_ext", "v_nl", "hartree", "exchange"]},
        "energy_gate": {"bound_Ha": 1e-6, "N128": gate128, "N160": gate160,
                        "note": "mixed = the energy the mixed path reports (FP64 terms of the FP32 orbitals); "
                                "fp32_operator = the FP32 operator's own terms, used by a mixed SCF only "
                                "while the energy moves by more than ~1e-4 Ha per iteration"},
        "force_ms": {"mixed": f32_ms, "fp64": f64_ms, "max_abs_dF_Ha_per_bohr": dF},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def _sync_time(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def run_workload(args):
    """Configuration workloads (one JSON line each); the headline metric is the default run."""
    import numpy as np
    import torch

    from gato_gb300.grid import Grid3D
    out = {"workload": args.workload}
    if args.workload == "batch48":
        # 48 seeded systems (H2 / LiH / HCl / H2O, 64^3..160^3, h 0.2..0.3), mixed precision,
        # concurrent streams vs one stream, FP64 continuation checks on the grids <= 96^3
        from gato_gb300.batch import draw_systems, fp64_check, solve_batch, summarize
        specs = draw_systems(48, seed=0)
        # warm-up (untimed): the process's first solve loads the library's kernels; both timed runs below
        # then build their own plans and projectors inside the timed region
        solve_batch(specs[:1], precision="mixed", streams=1, max_iters=2, tol=1e-7)
        res, wall = solve_batch(specs, precision="mixed", streams=args.streams, max_iters=80, tol=1e-7)
        out["concurrent"] = summarize(res, wall)
        out["concurrent"]["streams"] = args.streams
        if args.batch_sequential:
            res1, wall1 = solve_batch(specs, precision="mixed", streams=1, max_iters=80, tol=1e-7)
            out["sequential_wall_s"] = wall1
            out["concurrency_speedup"] = wall1 / wall
            # same kernels on the same inputs: the two runs must agree bit for bit
            out["bitwise_mismatches_vs_sequential"] = [
                a.spec.name for a, b in zip(res, res1)
                if a.point.energy != b.point.energy or not torch.equal(a.forces, b.forces)]
        checks = [fp64_check(r) for r in res if r.spec.N <= 96]
        both = [c for c in checks if c["fp64_converged"] and c["mixed_converged"]]
        out["fp64_checks"] = {"systems": len(checks), "both_converged": len(both),
                              "max_abs_dE_converged": max((c["abs_dE"] for c in both), default=None),
                              "max_abs_dF_same_orbitals": max(c["max_abs_dF"] for c in checks),
                              "per_system": checks}
        print(json.dumps(out), flush=True)
        return
    if args.workload == "hydrogen64":
        # hydrogen 64^3, L = 20, 7-point Laplacian, softened Coulomb a = 0.1, Lanczos m = 80, K = 1
        from gato_gb300.hamiltonian import Hamiltonian
        from gato_gb300.potentials import softened_coulomb
        from gato_gb300.solvers.lanczos import lanczos
        g = Grid3D(64, 20.0)
        psi0 = np.random.default_rng(0).uniform(0.0, 1.0, g.shape)
        for prec, dt in (("fp64", torch.float64), ("mixed", torch.float32)):
            H = Hamiltonian(g, softened_coulomb(g, 1.0, 0.1, dtype=dt), order=2)
            p = torch.tensor(psi0, device="cuda", dtype=dt)
            lanczos(H, p, 80, 1)
            res, dt_s = _sync_time(lambda: lanczos(H, p, 80, 1))
            out[prec] = {"E0": float(res.eigenvalues[0]), "lanczos_s": dt_s}
        out["abs_dE0"] = abs(out["mixed"]["E0"] - out["fp64"]["E0"])
    elif args.workload == "helium96":
        # helium RHF 96^3, L = 16, Z = 2, softening 0.1, Gaussian + 1e-3 noise, mixing 0.5; FP64 to tol 1e-8.
        # The mixed SCF's energy noise floor is ~1e-8..1e-7 Ha (FP64 energies of orbitals from the FP32 Fock
        # operator), so it stops at 1e-7 and an FP64 continuation from its orbitals goes on to 1e-8.
        from gato_gb300.potentials import softened_coulomb
        from gato_gb300.scf import scf_rhf, to_fields
        g = Grid3D(96, 16.0)
        X, Y, Z = (a.cpu().numpy() for a in g.coords())
        phi0 = np.exp(-(X * X + Y * Y + Z * Z)) + 1e-3 * np.random.default_rng(3).standard_normal(g.shape)
        Vc = softened_coulomb(g, 2.0, 0.1)

        def helium(prec, init, tol, iters=30):
            return scf_rhf(Vc, g, 1, initial_orbitals=init, max_iters=iters, tol=tol, mixing=0.5, order=4,
                           epsilon=0.1, precision=prec)
        for prec, dt, tol in (("mixed", torch.float32, 1e-7), ("fp64", torch.float64, 1e-8)):
            init = torch.tensor(phi0, device="cuda", dtype=dt)[..., None]
            # the process's first solve also loads the library's kernels and builds the plans (cold start):
            # timed apart, then the same solve again
            _, t_first = _sync_time(lambda: helium(prec, init, tol))
            r, t = _sync_time(lambda: helium(prec, init, tol))
            out[prec] = {"E": r.energy, "iters": r.n_iters, "converged": r.converged, "tol": tol, "scf_s": t,
                         "scf_s_first_call": t_first}
            if prec == "mixed":
                mixed_orbitals = r.orbitals
        rc, tc = _sync_time(lambda: helium("fp64", to_fields(mixed_orbitals, torch.float64).permute(1, 2, 3, 0),
                                           1e-8, args.fp64_iters + 5))
        out["fp64_continuation"] = {"E": rc.energy, "iters": rc.n_iters, "converged": rc.converged, "scf_s": tc}
        out["abs_dE"] = abs(out["mixed"]["E"] - out["fp64"]["E"])
        out["abs_dE_continuation"] = abs(rc.energy - out["fp64"]["E"])
    elif args.workload in ("water128", "water-geomopt"):
        from gato_gb300.physics.water import (bo_energy, hellmann_feynman_force, optimize_water_geometry,
                                              solve_rhf_at_geometry, water_hgh_elements, water_initial_geometry)
        from gato_gb300.scf import to_fields
        N, h = args.N, H_DEFAULT
        g = Grid3D(N, N * h)
        el = water_hgh_elements()
        rng = np.random.default_rng(11)
        if args.workload == "water128":
            nuc = water_initial_geometry(1.81, 104.5)
            nuc = type(nuc)(nuc.positions + torch.tensor(rng.uniform(-0.05, 0.05, (3, 3))), nuc.charges)
            # the mixed SCF's energy noise floor is ~1e-8..1e-7 Ha (FP64 energies of orbitals from the
            # FP32 Fock operator), so it stops at 1e-7; the FP64 continuation below goes to 1e-8
            # warm-up: the process's first solve loads the library's kernels and builds the plans
            _, t_cold = _sync_time(lambda: solve_rhf_at_geometry(nuc, el, g, precision="mixed", tol=1e-7,
                                                                 max_iters=2))
            out["first_call_2_iterations_s"] = t_cold
            p32, t32 = _sync_time(lambda: solve_rhf_at_geometry(nuc, el, g, precision="mixed", tol=1e-7,
                                                                max_iters=80))
            out["mixed"] = {"E": p32.energy, "iters": p32.n_iters, "converged": p32.converged, "scf_s": t32,
                            "orbital_energies": p32.orbital_energies.cpu().tolist()}
            # FP64 continuation from the mixed fixed point: same converged state if the paths agree
            p64, t64 = _sync_time(lambda: solve_rhf_at_geometry(
                nuc, el, g, precision="fp64", tol=1e-8, max_iters=args.fp64_iters,
                initial_orbitals=to_fields(p32.orbitals, torch.float64).permute(1, 2, 3, 0)))
            out["fp64_continuation"] = {"E": p64.energy, "iters": p64.n_iters, "converged": p64.converged,
                                        "scf_s": t64,
                                        "orbital_energies": p64.orbital_energies.cpu().tolist()}
            out["abs_dE"] = abs(p32.energy - p64.energy)
            # orbital energies move at first order with the density (the energy at second order), so
            # this difference includes the continuation's own SCF update, not only the precision
            out["max_abs_d_orbital_energy"] = float(
                (p32.orbital_energies.cpu() - p64.orbital_energies.cpu()).abs().max())
        else:
            R, ang = rng.uniform(1.5, 2.3), rng.uniform(90.0, 130.0)
            nuc = water_initial_geometry(R, ang)
            steps, worst, fd_ms = [], 0.0, 0.0
            d = 1e-3

            def fd_check(point):
                nonlocal worst, fd_ms
                F = hellmann_feynman_force(point, el, g).numpy()
                o64 = to_fields(point.orbitals).to(torch.float64).permute(1, 2, 3, 0)
                t0 = time.perf_counter()
                for a in range(3):
                    for c in range(3):
                        pp, pm = point.nuclei.positions.clone(), point.nuclei.positions.clone()
                        pp[a, c] += d
                        pm[a, c] -= d
                        fd = -(float(bo_energy(pp, point.nuclei.charges, o64, el, g))
                               - float(bo_energy(pm, point.nuclei.charges, o64, el, g))) / (2 * d)
                        worst = max(worst, abs(F[a, c] - fd))
                fd_ms += 1e3 * (time.perf_counter() - t0)

            from gato_gb300.geometry_opt import optimize_geometry_alternating
            from gato_gb300.physics.water import bo_grad_positions

            def solve_at(nuclei, prev):
                return solve_rhf_at_geometry(nuclei, el, g, precision="mixed",
                                             initial_orbitals=prev.orbitals if prev is not None else None)

            def on_step(step, p):
                steps.append(p.energy)
                if step % args.fd_every == 0 or step == args.geom_steps - 1:
                    fd_check(p)
            (final, traj), t = _sync_time(lambda: optimize_geometry_alternating(
                nuc, solve_at_geometry=solve_at, learning_rate=0.02, geom_steps=args.geom_steps,
                bo_grad=lambda p: bo_grad_positions(p.nuclei.positions, p.nuclei.charges, p.orbitals, el, g),
                on_step=on_step))
            _, tf = _sync_time(lambda: hellmann_feynman_force(final, el, g))
            out.update({"geom_steps": args.geom_steps, "opt_s_including_fd_checks": t,
                        "fd_check_s": fd_ms / 1e3, "E_first_last": [traj[0].energy, final.energy],
                        "max_abs_force_minus_fd_Ha_per_bohr": worst, "force_ms_mixed": 1e3 * tf,
                        "scf_iters_per_step": [p.n_iters for p in traj[1:]],
                        "final_R_OH": float(torch.linalg.norm(final.nuclei.positions[1] - final.nuclei.positions[0]))})
    print(json.dumps(out), flush=True)


def run_profile(args):
    """The block (or matvec) Fock apply alone, for ncu: no autotune sweep, no FP64, no CPU leg.

    One launch group spans every pair field (what the autotuner picks at 128^3).
    Prints one JSON line with the kernel launches of one step.
    """
    import torch

    from gato_gb300 import _lib
    from gato_gb300.autotune import set_plan
    from gato_gb300.geometry import Nuclei
    from gato_gb300.grid import Grid3D
    from gato_gb300.physics.water import water_hgh_elements
    from gato_gb300.pseudopotentials import hgh_local_potential, nonlocal_for
    from gato_gb300.scf import Operator, _density_fields, pair_fields
    from gato_gb300.solvers.poisson import get_plan

    dtype = torch.float32 if args.profile_dtype == "f32" else torch.float64
    N, h = args.N, H_DEFAULT
    g = Grid3D(N, N * h)
    pos, orbs = synthetic_water(N, h)
    nuc = Nuclei(torch.tensor(pos), torch.tensor([8.0, 1.0, 1.0], dtype=torch.float64))
    el = water_hgh_elements()
    fields = torch.tensor(orbs, device="cuda").to(dtype).contiguous()
    plan = get_plan(N, h, h / 2, dtype, pair_fields(N_OCC))
    set_plan(plan, plan.max_fields, args.engine)
    op = Operator(g, dtype, 4, "dirichlet")
    op.set_potential((hgh_local_potential(nuc, el, g, dtype) + plan.potential(_density_fields(fields))).contiguous())
    op.set_nonlocal(nonlocal_for(nuc, el, g, dtype))
    op.set_exchange(plan, fields)
    out = torch.empty_like(fields)
    if args.profile == "scf":
        # two mixed SCF iterations of the 128^3 water from the seeded orbitals (the C3 inner loop)
        from gato_gb300.physics.water import solve_rhf_at_geometry
        init = torch.tensor(orbs, device="cuda").permute(1, 2, 3, 0)
        step = lambda: solve_rhf_at_geometry(nuc, el, g, precision="mixed", max_iters=2,   # noqa: E731
                                             initial_orbitals=init)
    elif args.profile == "block":
        step = lambda: op.apply_block(out)   # noqa: E731
    else:
        step = lambda: op.apply(fields[0], out[0])   # noqa: E731
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    n0 = _lib.launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({"profile": args.profile, "dtype": args.profile_dtype, "N": N, "steps": args.steps,
                      "ms_per_step": 1e3 * dt / args.steps,
                      "launches_per_step": (_lib.launch_count() - n0) / args.steps}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--streams", type=int, default=8, help="concurrent streams of the 48-system batch")
    ap.add_argument("--batch-sequential", type=int, default=1, help="also time the 48-system batch on one stream")
    ap.add_argument("--workload", default=None,
                    choices=["hydrogen64", "helium96", "water128", "water-geomopt", "batch48"],
                    help="run one of the end-to-end workloads instead of the headline metric: hydrogen 64^3 "
                         "Lanczos, helium 96^3 SCF, water 128^3 SCF, water geometry optimisation, "
                         "48 mixed-size systems")
    ap.add_argument("--fp64-iters", type=int, default=3)
    ap.add_argument("--geom-steps", type=int, default=60)
    ap.add_argument("--fd-every", type=int, default=20)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gato", choices=["gato", "reference"])
    ap.add_argument("--N", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--profile", default=None, choices=["block", "matvec", "scf"],
                    help="run only the block / matvec Fock apply or two SCF iterations (for ncu captures)")
    ap.add_argument("--profile-dtype", default="f32", choices=["f32", "f64"])
    ap.add_argument("--engine", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="FFT engine of the --profile run (see gato_poisson_tune)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile:
        run_profile(args)
    elif args.workload:
        run_workload(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gato(args)


if __name__ == "__main__":
    main()
