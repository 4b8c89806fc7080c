"""Host-side logic of bench.py (no GPU): the clock record of the timed region and the
reference arm's JSON line on a small sample."""
import json
import subprocess
import sys
from pathlib import Path

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
