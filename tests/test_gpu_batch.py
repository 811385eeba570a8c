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
