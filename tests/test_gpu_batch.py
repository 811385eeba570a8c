"""The batched mixed-size workload (several molecules, grids and spacings, concurrent streams)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")


def test_batch_concurrent_equals_sequential_and_fp64():
    from gato_gb300.batch import draw_systems, fp64_check, solve_batch, summarize
    specs = draw_systems(6, seed=3, grids=(32, 40))
    assert {s.name.split("#")[0] for s in specs} >= {"H2", "HCl"}
    seq, _ = solve_batch(specs, streams=1, max_iters=60)
    par, wall = solve_batch(specs, streams=3, max_iters=60)
    assert len({r.stream for r in par}) > 1
    for a, b in zip(seq, par):
        assert a.spec.name == b.spec.name and a.point.converged
        # same kernels on the same inputs: concurrency must not change a bit
        assert a.point.energy == b.point.energy, a.spec.name
        assert torch.equal(a.forces, b.forces)
        assert bool(torch.isfinite(a.forces).all())
    summ = summarize(par, wall)
    assert summ["systems"] == 6 and summ["converged"] == 6 and summ["systems_per_s"] > 0
    # The mixed SCF's FP64 energies of FP32 orbitals fluctuate by ~1e-8..5e-7 Ha per iteration on these
    # 32^3-40^3 boxes, so it stops at 1e-7; the FP64 continuation in fp64_check goes to 1e-9
    tight, _ = solve_batch(specs[:2], streams=2, max_iters=80, tol=1e-7)
    for r in tight:
        chk = fp64_check(r)
        assert chk["finite"] and chk["mixed_converged"] and chk["fp64_converged"], chk
        assert chk["abs_dE"] < 1e-6 and chk["max_abs_dF"] < 1e-5, chk


def test_batch_worker_error_surfaces():
    """A failing system stops the pool and its exception reaches the caller (odd electron count)."""
    from gato_gb300.batch import SystemSpec, draw_systems, solve_batch
    from gato_gb300.geometry import Nuclei
    from gato_gb300.pseudopotentials import lookup
    good = draw_systems(1, seed=0, grids=(32,))[0]
    pos = torch.tensor([[0.0, 0.0, -1.0], [0.0, 0.0, 0.0], [0.0, 0.0, 1.0]], dtype=torch.float64)
    bad = SystemSpec("H3", Nuclei(pos, torch.ones(3, dtype=torch.float64)), 32, 0.25, (lookup("H"),) * 3)
    with pytest.raises(ValueError):
        solve_batch([good, bad], streams=2, max_iters=5)


def test_threads_on_packed_shapes_are_bitwise_stable():
    """Four threads, each on its own stream, drive FP32 operators on 64^3 and 96^3 grids (the
    packed column passes, the persistent z forward, the stencil's TMA ring and the cluster
    non-local apply all run concurrently on shared SMs). Every apply, block apply and energy-term
    evaluation must equal the single-threaded result bit for bit: a shared-memory buffer that a
    copy engine refills while another kernel's loads still queue behind it would show up here."""
    import threading
    from gato_gb300 import scf
    from gato_gb300.batch import draw_systems
    from gato_gb300.solvers.poisson import get_plan
    f32 = torch.float32
    specs = draw_systems(10, seed=0, grids=(64, 96))
    picked = [next(s for s in specs if s.N == 96 and s.n_occ() == 4),
              next(s for s in specs if s.N == 64 and s.n_occ() == 4)]
    gen = torch.Generator(device="cuda").manual_seed(11)
    cases = []
    for sp in picked:
        shape = sp.grid.shape
        cases.append((sp, torch.randn(shape, device="cuda", dtype=f32, generator=gen),
                      torch.randn(shape, device="cuda", dtype=f32, generator=gen),
                      0.01 * torch.randn((4,) + shape, device="cuda", dtype=f32, generator=gen),
                      torch.randn(shape, device="cuda", dtype=f32, generator=gen)))

    def run(case, overlap):
        sp, V, Vx, orb, psi = case
        model, grid = sp.model(), sp.grid
        nl = scf._native_nl(model.nonlocal_op(sp.nuclei, grid, f32), grid, f32)
        op = scf.Operator(grid, f32)
        op.overlap(overlap)
        op.set_nonlocal(nl)
        op.set_potential(V)
        op.set_exchange(get_plan(grid.N, grid.h, model.epsilon(grid), f32, scf.pair_fields(4)), orb)
        return [op.apply(psi), op.apply_block(), op.energy_terms(Vx)], op

    refs = []
    for c in cases:
        outs, _ = run(c, True)
        torch.cuda.synchronize()
        refs.append([t.clone() for t in outs])
    mismatches, errors = [], []

    def worker(k):
        try:
            s = torch.cuda.Stream()
            keep, outs = [], []
            with torch.cuda.stream(s):
                for i in range(12):
                    ci = (i + k) % len(cases)
                    r, op = run(cases[ci], overlap=(i // 2) % 2 == 0)
                    keep.append(op)
                    outs.append((ci, r))
                s.synchronize()
            for ci, r in outs:
                for j, name in enumerate(("apply", "block", "energy")):
                    if not torch.equal(r[j], refs[ci][j]):
                        mismatches.append((k, picked[ci].name, name))
        except BaseException as e:   # reported after the join
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    assert not errors, errors
    assert not mismatches, mismatches[:8]


def test_batch_mixed_64_128_concurrent_equals_sequential():
    """The batch on 64^3 and 128^3 grids (packed column passes, persistent z forward, one-sweep
    Lanczos with its side stream, cluster projectors): four systems on three streams give the same
    energies and forces bit for bit as on one stream, and every energy and force is finite."""
    from gato_gb300.batch import draw_systems, solve_batch
    specs = draw_systems(4, seed=4, grids=(64, 128))
    assert sorted(s.N for s in specs) == [64, 64, 128, 128]
    seq, _ = solve_batch(specs, streams=1, max_iters=12, tol=1e-6)
    par, _ = solve_batch(specs, streams=3, max_iters=12, tol=1e-6)
    assert len({r.stream for r in par}) > 1
    for a, b in zip(seq, par):
        assert a.spec.name == b.spec.name
        assert a.point.energy == b.point.energy, a.spec.name
        assert torch.equal(a.forces, b.forces), a.spec.name
        assert torch.isfinite(torch.as_tensor(a.point.energy)) and bool(torch.isfinite(a.forces).all())
