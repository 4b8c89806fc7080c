#!/usr/bin/env python
"""Benchmark: SyMBA body-steps/s on one GB300 for the C1 disk (2000 massive bodies
+ 10 000 test particles, 1-Hill-radius encounter radius, dt = 0.005 yr).

A step is one symba_step_system call on the device-resident system.  The
headline ``value`` is the mixed-precision path (FP32 pair kicks with float-float
sums; FP64 drift, encounter tests and recursion); the FP64 path runs the same
steps from the same initial conditions and is reported beside it together with
both paths' |dE/E| and |dL/L| (matched-accuracy comparison).

Timing: W untimed warm-up steps, then K steps, each preceded by an untimed
512 MB memset that evicts L2 (the C1 working set, ~3 MB, would otherwise sit in
L2), each bracketed by CUDA events on the library's stream.  Under torchrun the
ranks run independent replicas (SyMBA does not shard across GPUs here) with a
barrier and the max time over ranks.

``--impl reference`` times the CPU restatement of the reference (the oracle,
OpenMP) on the same workload on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SyMBA body-steps/s on 1 GB300: mixed+batched vs FP64 GPU at matched |ΔE/E|"
UNIT = "body-steps/s"
FLOPS_PER_INTERACTION = 20.0  # GPU Gems 3 ch. 31 convention (sqrt and divide count 1)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--npl", type=int, default=2000)
    p.add_argument("--ntp", type=int, default=10000)
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    return p.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group(backend="gloo")
        pg = td
    return world, rank, local, pg


def workload(args):
    from swiftest_gb300 import initial_conditions as IC
    cfg = dict(IC.CONFIGS["C1"])
    cfg["npl"], cfg["ntp"] = args.npl, args.ntp
    cb, pl, tp = IC.make_system(seed=cfg["seed"], npl=cfg["npl"], ntp=cfg["ntp"], mmin=cfg["mmin"], mmax=cfg["mmax"],
                                amin=cfg["amin"], amax=cfg["amax"], sig_e=cfg["sig_e"], sig_i=cfg["sig_i"])
    pl = IC.sort_for_integrator(pl, "SYMBA")
    return cfg, cb, pl, tp


def config_block(cfg, precision):
    return {"workload": f"C1 SyMBA disk: {cfg['npl']} pl + {cfg['ntp']} tp, a in [{cfg['amin']}, {cfg['amax']}] AU, "
                        f"RHSCALE={cfg['rhscale']} (1 Hill radius), dt={cfg['dt']} yr, TRIANGULAR encounter checks",
            "npl": cfg["npl"], "ntp": cfg["ntp"], "dt": cfg["dt"], "rhscale": cfg["rhscale"], "seed": cfg["seed"],
            "precision": precision, "l2": "flushed before every timed step (512 MB memset, untimed)"}


class ClockSampler:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def rel_energy(e0, e1):
    dE = abs(e1["te_helio"] - e0["te_helio"]) / abs(e0["te_helio"])
    dE_ref = abs(e1["te"] - e0["te"]) / abs(e0["te"])
    dL = float(np.linalg.norm(e1["L"] - e0["L"]) / np.linalg.norm(e0["L"]))
    return dE, dE_ref, dL


def run_path(ctx, cfg, cb, pl, tp, precision, steps, warmup, profile=False, clocks=None):
    from swiftest_gb300.api import NBodySystem
    s = NBodySystem(ctx, "SYMBA", cb, pl, tp, dt=cfg["dt"], rhscale=cfg["rhscale"], lclose=True, precision=precision)
    e0 = s.energy()
    s.step(warmup)
    ctx.synchronize()
    launches0 = ctx.launches
    if profile:
        s.profile(True)
    total_ms = 0.0
    cm = clocks if clocks is not None else _Null()
    with cm:
        for _ in range(steps):
            ctx.flush_l2()
            ctx.event_record(0)
            s.step(1)
            ctx.event_record(1)
            total_ms += ctx.event_elapsed_ms(0, 1)
    launches = ctx.launches - launches0  # kernels of ours (the L2-flush memsets are not counted)
    prof = s.profile_read() if profile else None
    if profile:
        s.profile(False)
    e1 = s.energy()
    stats = s.stats()
    s.close()
    return total_ms, launches, prof, rel_energy(e0, e1), stats


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def run_e2e(ctx, cfg, cb, pl, tp, precision, steps):
    """Same metric through the C ABI with host buffers: every step uploads the
    state (pinned host arrays -> device), steps once, and reads the state back."""
    import torch
    from swiftest_gb300.api import NBodySystem
    s = NBodySystem(ctx, "SYMBA", cb, pl, tp, dt=cfg["dt"], rhscale=cfg["rhscale"], lclose=True, precision=precision)
    s.step(2)
    npl, ntp = s.npl, s.ntp
    pinned = [torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy() for n in (npl, npl, ntp, ntp)]
    s.get_state_async(*pinned)
    ctx.synchronize()
    total_ms = 0.0
    for _ in range(steps):
        ctx.flush_l2()
        ctx.event_record(2)
        s.set_state(*pinned)
        s.step(1)
        s.get_state_async(*pinned)
        ctx.event_record(3)
        total_ms += ctx.event_elapsed_ms(2, 3)
    s.close()
    nbytes = sum(a.nbytes for a in pinned)
    return total_ms, nbytes


def cpu_baseline(cfg, cb, pl, tp, budget_s):
    """The oracle (C restatement of the reference's OpenMP path) on this host: steps of
    the same C1 system until the time budget is used."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    s = O.OracleSystem("SYMBA", cb, pl, tp, dt=cfg["dt"], rhscale=cfg["rhscale"], lclose=True)
    s.step(1)
    n, t0 = 0, time.perf_counter()
    while True:
        s.step(1)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 200:
            break
    nb = cfg["npl"] + cfg["ntp"]
    return {"value": nb * n / el, "unit": UNIT, "cores": int(os.environ.get("OMP_NUM_THREADS", threads)),
            "kind": "port",
            "sample": f"{n} SyMBA steps of the same C1 system ({nb} bodies) after 1 warm-up step, "
                      f"{el:.1f} s wall, C restatement of the reference loops with OpenMP"}


def reference_arm(args, world, rank):
    if rank != 0:
        return 0
    cfg, cb, pl, tp = workload(args)
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    s = O.OracleSystem("SYMBA", cb, pl, tp, dt=cfg["dt"], rhscale=cfg["rhscale"], lclose=True)
    s.step(max(args.warmup, 1))
    t0 = time.perf_counter()
    s.step(args.steps)
    el = time.perf_counter() - t0
    nb = cfg["npl"] + cfg["ntp"]
    v = nb * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded C1 disk)",
            "config": config_block(cfg, "FP64 CPU"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                             "sample": f"{args.steps} timed SyMBA steps of the full C1 system after {args.warmup} "
                                       "warm-up steps (C restatement of the reference's OpenMP loops; the Fortran "
                                       "reference cannot be compiled on this image)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def load_traffic():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except json.JSONDecodeError:
            return {}
    return {}


def main():
    args = parse()
    world, rank, local, td = dist_setup(args)
    if args.impl == "reference":
        return reference_arm(args, world, rank)
    from swiftest_gb300 import build as B
    B.build()
    from swiftest_gb300.api import Context
    cfg, cb, pl, tp = workload(args)
    ctx = Context(local)
    nb = cfg["npl"] + cfg["ntp"]
    clocks = ClockSampler(local)
    if td:
        td.barrier()
    ms_mixed, launches, prof, (dE_m, dEr_m, dL_m), st_m = run_path(ctx, cfg, cb, pl, tp, "MIXED", args.steps,
                                                                    args.warmup, profile=True, clocks=clocks)
    ms_fp64, _, prof64, (dE_f, dEr_f, dL_f), st_f = run_path(ctx, cfg, cb, pl, tp, "FP64", args.steps, args.warmup,
                                                             profile=True)
    if td:
        import torch
        t = torch.tensor([ms_mixed, ms_fp64], dtype=torch.float64)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        ms_mixed, ms_fp64 = float(t[0]), float(t[1])
    e2e_ms, e2e_bytes = run_e2e(ctx, cfg, cb, pl, tp, "MIXED", args.steps)
    value = world * nb * args.steps / (ms_mixed * 1e-3)
    fp64_value = world * nb * args.steps / (ms_fp64 * 1e-3)

    # roofline of the dominant kernel class (mixed path), from the live CUDA-event profile
    npl, ntp = cfg["npl"], cfg["ntp"]
    flops_per_launch = {"kick_pl": FLOPS_PER_INTERACTION * npl * (npl - 1),
                        "kick_tp": FLOPS_PER_INTERACTION * npl * ntp}
    dom = max(prof, key=lambda k: prof[k]["ms"])
    roof = None
    peak32 = ctx.probe_peak_tflops("fp32")
    peak64 = ctx.probe_peak_tflops("fp64")
    traffic = load_traffic()
    kick_cls = max(("kick_pl", "kick_tp"), key=lambda k: prof[k]["ms"])
    if prof[kick_cls]["launches"]:
        avg_ms = prof[kick_cls]["ms"] / prof[kick_cls]["launches"]
        ach = flops_per_launch[kick_cls] / (avg_ms * 1e-3) / 1e12
        roof = {"kernel": f"{kick_cls} (mixed FP32 pair kick)", "bound": "fp32", "achieved": ach, "peak": peak32,
                "unit": "TFLOP/s", "frac": ach / peak32 if peak32 else None,
                "peak_source": "FP32 FFMA-chain probe measured by bench.py on this GPU (MEASURED_PEAKS.json "
                               "has no FP32 figure)",
                "algorithmic_flops_per_launch": flops_per_launch[kick_cls], "avg_launch_ms": avg_ms,
                "traffic": traffic.get(kick_cls)}
    kernel_profile = {k: {"launches": v["launches"], "ms_total": round(v["ms"], 4),
                          "share": round(v["ms"] / ms_mixed, 4)} for k, v in prof.items()}
    cpu = cpu_baseline(cfg, cb, pl, tp, args.cpu_seconds) if rank == 0 else None
    csum = clocks.summary()
    pairs_per_step = 2 * (npl * (npl - 1) + npl * ntp)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_mixed / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (f32 pair kicks)", "data": "synthetic (seeded C1 disk, numpy default_rng)",
        "config": config_block(cfg, "mixed"),
        "fp64_path": {"value": fp64_value, "ms_per_step": ms_fp64 / args.steps, "dE_E": dE_f, "dE_E_ref_formula": dEr_f,
                      "dL_L": dL_f, "stats": st_f,
                      "kernel_profile": {k: {"launches": v["launches"], "ms_total": round(v["ms"], 4)}
                                         for k, v in prof64.items()}},
        "mixed_path": {"dE_E": dE_m, "dE_E_ref_formula": dEr_m, "dL_L": dL_m, "stats": st_m},
        "speedup_mixed_vs_fp64": value / fp64_value,
        "pair_interactions_per_s": pairs_per_step * args.steps / (ms_mixed * 1e-3),
        "kernel_profile": kernel_profile, "dominant_kernel_class": dom,
        "roofline": roof, "fp64_peak_probe_tflops": peak64,
        "cpu_baseline": cpu,
        "clocks": csum,
        "e2e": {"value": world * nb * args.steps / (e2e_ms * 1e-3), "unit": UNIT,
                "h2d_bytes_per_step": e2e_bytes // 2, "d2h_bytes_per_step": e2e_bytes // 2},
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if td:
        td.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
