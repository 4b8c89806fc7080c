"""Host-side logic of bench.py (no GPU): the clock record of the timed region and the
reference arm's JSON line on a small sample."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

import bench

ROOT = Path(__file__).resolve().parents[1]


def _row(sm, power, reasons=("Not Active",) * 4):
    return ["0", str(sm), "2070", str(power), "0x0", *reasons]


def test_clock_summary_keeps_the_timed_region():
    cs = bench.ClockSampler(0)
    cs.rows = [_row(1000, 300),  # before the timed region (idle clocks)
               _row(2070, 900, ("Not Active", "Not Active", "Not Active", "Active")),
               _row(2065, 950),
               _row(1000, 200, ("Not Active", "Active", "Not Active", "Not Active"))]  # after it
    cs.i0, cs.i1 = 1, 3
    s = cs.summary()
    assert s["samples"] == 2 and s["samples_in_timed_region"] == 2
    assert s["sm_mhz"] == 2067.5 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_without_samples_in_the_region():
    # a timed region shorter than the sampling interval falls back to the samples around it
    cs = bench.ClockSampler(0)
    cs.rows = [_row(2070, 900), _row(2060, 900)]
    cs.i0 = cs.i1 = 1
    s = cs.summary()
    assert s["samples_in_timed_region"] == 0 and s["samples"] == 2 and s["reasons"] == []


def test_clock_summary_without_nvidia_smi():
    s = bench.ClockSampler(0).summary()
    assert s["sm_mhz"] is None and s["reasons"] == ["nvidia-smi unavailable"]


def test_reference_arm_line():
    # the reference arm (the C restatement on the host cores) prints one JSON line with the
    # contract's keys; one bounded C1 sample
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "c1",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([x for x in out.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "body-steps/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def _rank_worker(rank, world, port, q):
    import os
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    td.barrier()
    # rank r took (r + 1) * 10 ms for its mixed steps and 5 ms for its FP64 steps
    ms = bench.max_over_ranks(td, [10.0 * (rank + 1), 5.0])
    q.put((rank, ms, bench.whole_job_rate(world, 1000, 4, ms[0])))
    td.destroy_process_group()


def test_replicas_take_the_slowest_rank_gloo():
    """--gpus N runs N independent replicas (torchrun ranks, gloo): every rank sees the max of
    the ranks' times, and the whole-job rate counts every rank's units over that time."""
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in res:
        assert ms == [20.0, 5.0]
        assert rate == 2 * 1000 * 4 / 20e-3


def test_gpus_must_match_world_size(monkeypatch):
    import argparse
    import pytest
    monkeypatch.setenv("WORLD_SIZE", "1")
    with pytest.raises(SystemExit):
        bench.dist_setup(argparse.Namespace(gpus=2))
    assert bench.dist_setup(argparse.Namespace(gpus=1))[0] == 1


def test_traffic_record_is_used_only_for_its_kick_shape(tmp_path, monkeypatch):
    # the recorded DRAM bytes of a capture go into the roofline line only when the run used
    # the kick shape that the capture ran
    (tmp_path / "profiles").mkdir()
    shape = {"plpl_tile": 128, "plpl_strip": 4, "plpl_warps_per_block": 2, "plpl_row_group": 2}
    rec = {"kick_pl_c4": {"bytes_per_launch": 49.1e6, "commit": "abc", "command": "ncu ...", "note": "n",
                          "plan": shape}}
    (tmp_path / "profiles" / "traffic.json").write_text(json.dumps(rec))
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    b, src = bench.load_traffic("kick_pl_c4", dict(shape, plpl="symmetric", pltp_shape=-1))
    assert b == 49.1e6 and src["commit"] == "abc"
    b, src = bench.load_traffic("kick_pl_c4", dict(shape, plpl_row_group=1, plpl_warps_per_block=1))
    assert b is None and "another kick shape" in src["note"]
    assert bench.load_traffic("kick_pl_c1", shape) == (None, None)


@pytest.mark.parametrize("workload", ["c4", "c3", "c3w", "c1"])
def test_workloads_make_their_system(monkeypatch, workload):
    # every workload builds its system through the public API classes, with or without a
    # forced symmetric-kick shape (recorded here by a stand-in class instead of the GPU)
    import swiftest_gb300.api as api
    calls = []

    class Fake:
        def __init__(self, *a, **k):
            calls.append(("new", k.get("precision")))

        def __getattr__(self, name):
            return lambda *a, **k: calls.append((name, a))

    monkeypatch.setattr(api, "Ensemble", Fake)
    monkeypatch.setattr(api, "NBodySystem", Fake)
    for shape in (None, "128,4,1,2"):
        argv = ["--workload", workload, "--nsys", "3"] + (["--kick-shape", shape] if shape else [])
        monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
        args = bench.parse()
        wl = {"c4": bench.C4, "c3": bench.C3, "c3w": bench.C3W, "c1": bench.C1}[workload](args)
        calls.clear()
        wl.make(None, "MIXED")
        assert calls[0] == ("new", "MIXED")
        forced = [c for c in calls if c[0] == "set_kick_group"]
        assert forced == ([("set_kick_group", (2,))] if shape and workload == "c4" else [])
