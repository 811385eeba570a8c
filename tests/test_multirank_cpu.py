"""The replicas path of `bench.py --gpus N` on CPU: world_size-2 gloo ranks agree on the
whole-job rate (every rank's steps over the slowest rank's time)."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    rate, t_job = bench.job_rate(1.0 + rank, 10, world, dist, "cpu")
    q.put((rank, rate, t_job, bench.dist_env()))
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, t_job, env in out:
        assert t_job == pytest.approx(2.0)          # the slower rank's time
        assert rate == pytest.approx(2 * 10 / 2.0)  # both ranks' steps over it
        assert env[0] == rank and env[1] == 2


def test_job_rate_single_rank_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(0.5, 10, 1) == (20.0, 0.5)
