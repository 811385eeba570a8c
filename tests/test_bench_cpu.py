"""Host logic of bench.py that runs without a GPU: the reference arm's JSON line
(the oracle port of the reference's block Fock apply on the host cores), its
rank-0-only rule under a multi-rank launch, and the clock sampler's summary."""
import argparse
import json

import bench


def _args(**kw):
    a = dict(N=16, steps=1, warmup=0, impl="reference", gpus=1)
    a.update(kw)
    return argparse.Namespace(**a)


def test_reference_arm_line(capsys, monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    bench.run_reference(_args())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["workload"] == bench.workload_name(16, bench.H_DEFAULT)
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_do_no_work(capsys, monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    bench.run_reference(_args())
    assert capsys.readouterr().out == ""


def test_clock_sampler_summary(tmp_path):
    cs = bench.ClockSampler(0)
    cs.path = str(tmp_path / "clocks.csv")
    cs.proc = object()   # as if nvidia-smi had run
    with open(cs.path, "w") as f:
        f.write("0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active\n")
        f.write("0, 1900, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n")
        f.write("garbage line\n")
    s = cs.summary()
    assert s == {"sm_mhz": 1985.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 2}


def test_clock_sampler_without_nvidia_smi():
    cs = bench.ClockSampler(0)
    assert cs.summary()["reasons"] == ["nvidia-smi unavailable"]
