#!/usr/bin/env python
"""Benchmark: SyMBA body-steps/s on one GB300, mixed precision + batched vs the FP64 GPU path.

Workload (default ``--workload c4``): the batched planetesimal-disk ensemble, 256
independent SyMBA systems with N_pl log-uniform in [500, 5000] (547,900 massive bodies in
total for seed 0), masses log-uniform in [1e-11, 1e-7] Msun, a in [0.5, 2] AU, e and i
Rayleigh(0.02), dt = 0.002 yr, 1-Hill-radius encounter radius (RHSCALE = 1), TRIANGULAR
level-0 checks, recursive encounter kicks in FP64.  A step advances every system by one
symba_step_system.  ``--workload c1`` runs the single-system C1 disk (2000 pl + 10 000 tp)
instead, ``--workload c3`` the batched HELIO ensemble (512 systems with test particles),
``--workload c3w`` the same systems stepped by WHM.

``value``: body-steps/s of the mixed-precision batched path (FP32 pair kicks with
float-float sums; FP64 drift, encounter decisions, recursion) with the state resident in
HBM.  The FP64 path (same kernels' FP64 variants, bit-identical to the reference loop
order) runs the same warm-up and timed steps from the same initial conditions; both
paths' |dE/E| and |dL/L| over those steps are reported (matched-accuracy comparison).

Timing: W untimed warm-up steps, then K steps, each preceded by an untimed 512 MB memset
that evicts L2 (the C4 state, ~60 MB, would otherwise sit in the 129 MB L2), each bracketed
by CUDA events on the library's stream.  A few more steps then run under the per-class
CUDA-event profile (kernel_profile, roofline); profiling serialises the step, so those
steps are not part of the timed value.  Under torchrun the ranks run independent replicas
(weak scaling; an ensemble shards by system with no exchange) with a barrier and the max
time over ranks.

``--impl reference`` times the CPU restatement of the reference (the oracle, OpenMP) on a
bounded sample of the same workload on rank 0.
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
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="c4", choices=["c4", "c3", "c3w", "c1"])
    p.add_argument("--nsys", type=int, default=None, help="first NSYS systems of the C4 ensemble")
    p.add_argument("--kick-shape", type=lambda v: tuple(int(x) for x in v.split(",")), default=None,
                   metavar="TILE,STRIP,WARPS,GROUP",
                   help="C4: force the symmetric pl-pl kick's shape (default: autotuned), e.g. 128,4,1,1")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    p.add_argument("--encounter", default="triangular", choices=["triangular", "sortsweep"],
                   help="mode of the SyMBA level-0 pl-pl and pl-tp checks (c4, c1)")
    return p.parse_args()


def dist_setup(args):
    """Ranks of a torchrun launch: one independent replica of the workload per GPU (the
    ensemble shards by system with no exchange), joined only by a gloo barrier and the max
    of the timings.  --gpus must equal the launch's WORLD_SIZE."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.gpus != world:
        raise SystemExit(f"--gpus {args.gpus} but WORLD_SIZE={world}: launch N>1 with "
                         f"python -m torch.distributed.run --nproc-per-node {args.gpus} bench.py --gpus {args.gpus}")
    pg = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group(backend="gloo")
        pg = td
    return world, rank, local, pg


def max_over_ranks(td, values):
    """The slowest rank's time for each entry of `values` (ms); identity without a group."""
    if td is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return [float(x) for x in t]


def whole_job_rate(world, units_per_rank, steps, ms):
    """Units per second of the whole job: every rank processed units_per_rank per step, and
    the job took the slowest rank's time."""
    return world * units_per_rank * steps / (ms * 1e-3)


# ---------------------------------------------------------------- workloads
class C4:
    """The batched SyMBA ensemble (CSR-packed systems stepped together)."""

    def __init__(self, args):
        from swiftest_gb300 import initial_conditions as IC
        self.E = IC.make_ensemble("C4", nsys=args.nsys)
        self.nbodies = int(self.E["npl"].sum() + self.E["ntp"].sum())
        self.plpl_pairs = float(sum(int(n) * (int(n) - 1) for n in self.E["npl"]))  # per kick evaluation
        self.pairs_per_step = 2 * self.plpl_pairs
        self.enc = getattr(args, "encounter", "triangular").upper()
        self.kick_shape = getattr(args, "kick_shape", None)

    def make(self, ctx, precision):
        from swiftest_gb300.api import Ensemble
        kw = {} if self.enc == "TRIANGULAR" else dict(encounter_check_plpl=self.enc, encounter_check_pltp=self.enc)
        ens = Ensemble(ctx, self.E, precision=precision, **kw)
        shape = getattr(self, "kick_shape", None)
        if shape and precision == "MIXED":  # forced symmetric-kick shape (else autotuned)
            tile, strip, warps, group = shape
            ens.set_kick_tile(tile)
            ens.set_kick_strip(strip)
            ens.set_kick_warps(warps)
            ens.set_kick_group(group)
        return ens

    def state_arrays(self):
        E = self.E
        return [(int(E["npl"].sum()), 3), (int(E["npl"].sum()), 3), (int(E["ntp"].sum()), 3), (int(E["ntp"].sum()), 3)]

    def config(self, precision):
        n = self.E["npl"]
        return {"workload": f"C4 batched SyMBA ensemble: {len(n)} planetesimal disks, N_pl log-uniform in "
                            f"[500, 5000] ({int(n.sum())} pl total, 0 tp), m in [1e-11, 1e-7] Msun, a in [0.5, 2] AU, "
                            f"e,i Rayleigh(0.02), dt=0.002 yr, RHSCALE=1.0 (1 Hill radius), {self.enc} level-0 checks",
                "nsys": len(n), "npl_total": int(n.sum()), "ntp_total": int(self.E["ntp"].sum()),
                "npl_min": int(n.min()), "npl_max": int(n.max()), "dt": self.E["dt"], "rhscale": self.E["rhscale"],
                "seed": 0, "precision": precision, "l2": "flushed before every timed step (512 MB memset, untimed)"}

    def oracle_sample(self, budget_s, steps_per_system=1):
        """Oracle steps over systems 0, 1, ... until the time budget is used."""
        from oracle import oracle as O
        from swiftest_gb300 import initial_conditions as IC
        cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
        bs, t_all, nsys = 0, 0.0, 0
        for pl, tp in self.E["systems"]:
            s = O.OracleSystem("SYMBA", cb, pl, None, dt=self.E["dt"], rhscale=self.E["rhscale"], lclose=True,
                               encounter_check_plpl=self.enc, encounter_check_pltp=self.enc)
            t0 = time.perf_counter()
            s.step(steps_per_system)
            t_all += time.perf_counter() - t0
            bs += len(pl["Gmass"]) * steps_per_system
            nsys += 1
            if t_all > budget_s:
                break
        return bs, t_all, f"{steps_per_system} SyMBA step(s) of each of the first {nsys} C4 systems ({bs} body-steps)"


class C3(C4):
    """The batched HELIO ensemble: 512 systems, N_pl log-uniform in [10, 2000], N_tp = 5 N_pl."""

    def __init__(self, args):
        from swiftest_gb300 import initial_conditions as IC
        self.enc = "TRIANGULAR"  # HELIO checks no encounters
        self.E = IC.make_ensemble("C3", nsys=args.nsys)
        self.nbodies = int(self.E["npl"].sum() + self.E["ntp"].sum())
        n = [int(x) for x in self.E["npl"]]
        self.plpl_pairs = float(sum(k * (k - 1) for k in n))
        self.pairs_per_step = 2 * float(sum(k * (k - 1) + 5 * k * k for k in n))

    def config(self, precision):
        n, m = self.E["npl"], self.E["ntp"]
        return {"workload": f"C3 batched HELIO ensemble: {len(n)} systems, N_pl log-uniform in [10, 2000] "
                            f"({int(n.sum())} pl, {int(m.sum())} tp = 5 N_pl), m in [1e-10, 1e-6] Msun, a in [0.5, 5] AU, "
                            "e Rayleigh(0.01), i Rayleigh(0.005), dt=0.01 yr, close-approach discards on",
                "nsys": len(n), "npl_total": int(n.sum()), "ntp_total": int(m.sum()), "dt": self.E["dt"], "seed": 0,
                "precision": precision, "l2": "flushed before every timed step (512 MB memset, untimed)"}

    def oracle_sample(self, budget_s, steps_per_system=1):
        from oracle import oracle as O
        from swiftest_gb300 import initial_conditions as IC
        cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
        bs, t_all, nsys = 0, 0.0, 0
        for pl, tp in self.E["systems"]:
            s = O.OracleSystem("HELIO", cb, pl, tp, dt=self.E["dt"], lclose=True)
            t0 = time.perf_counter()
            s.step(steps_per_system)
            t_all += time.perf_counter() - t0
            bs += (len(pl["Gmass"]) + len(tp["rh"])) * steps_per_system
            nsys += 1
            if t_all > budget_s:
                break
        return bs, t_all, f"{steps_per_system} HELIO step(s) of each of the first {nsys} C3 systems ({bs} body-steps)"


class C3W(C3):
    """The batched WHM ensemble: the C3 systems stepped by WHM (Jacobi coordinates)."""

    def __init__(self, args):
        from swiftest_gb300 import initial_conditions as IC
        self.enc = "TRIANGULAR"  # WHM checks no encounters
        self.E = IC.make_ensemble("C3", nsys=args.nsys, integrator="WHM")
        self.nbodies = int(self.E["npl"].sum() + self.E["ntp"].sum())
        n = [int(x) for x in self.E["npl"]]
        self.plpl_pairs = float(sum(k * (k - 1) for k in n))
        self.pairs_per_step = float(sum(k * (k - 1) + 5 * k * k for k in n))  # one evaluation per step

    def config(self, precision):
        c = super().config(precision)
        c["workload"] = c["workload"].replace("C3 batched HELIO ensemble", "C3 batched WHM ensemble")
        return c

    def oracle_sample(self, budget_s, steps_per_system=1):
        from oracle import oracle as O
        from swiftest_gb300 import initial_conditions as IC
        cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
        bs, t_all, nsys = 0, 0.0, 0
        for pl, tp in self.E["systems"]:
            s = O.OracleSystem("WHM", cb, pl, tp, dt=self.E["dt"], lclose=True)
            t0 = time.perf_counter()
            s.step(steps_per_system)
            t_all += time.perf_counter() - t0
            bs += (len(pl["Gmass"]) + len(tp["rh"])) * steps_per_system
            nsys += 1
            if t_all > budget_s:
                break
        return bs, t_all, f"{steps_per_system} WHM step(s) of each of the first {nsys} C3 systems ({bs} body-steps)"


class C1:
    """The single-system C1 disk."""

    def __init__(self, args):
        from swiftest_gb300 import initial_conditions as IC
        cfg = dict(IC.CONFIGS["C1"])
        cb, pl, tp = IC.make_system(seed=cfg["seed"], npl=cfg["npl"], ntp=cfg["ntp"], mmin=cfg["mmin"],
                                    mmax=cfg["mmax"], amin=cfg["amin"], amax=cfg["amax"], sig_e=cfg["sig_e"],
                                    sig_i=cfg["sig_i"])
        self.cfg, self.cb, self.pl, self.tp = cfg, cb, IC.sort_for_integrator(pl, "SYMBA"), tp
        self.nbodies = cfg["npl"] + cfg["ntp"]
        npl, ntp = cfg["npl"], cfg["ntp"]
        self.plpl_pairs = float(npl * (npl - 1))
        self.pairs_per_step = 2.0 * (npl * (npl - 1) + npl * ntp)
        self.enc = getattr(args, "encounter", "triangular").upper()

    def make(self, ctx, precision):
        from swiftest_gb300.api import NBodySystem
        c = self.cfg
        return NBodySystem(ctx, "SYMBA", self.cb, self.pl, self.tp, dt=c["dt"], rhscale=c["rhscale"], lclose=True,
                           precision=precision, encounter_check_plpl=self.enc, encounter_check_pltp=self.enc)

    def state_arrays(self):
        n, m = self.cfg["npl"], self.cfg["ntp"]
        return [(n, 3), (n, 3), (m, 3), (m, 3)]

    def config(self, precision):
        c = self.cfg
        return {"workload": f"C1 SyMBA disk: {c['npl']} pl + {c['ntp']} tp, a in [{c['amin']}, {c['amax']}] AU, "
                            f"RHSCALE={c['rhscale']} (1 Hill radius), dt={c['dt']} yr, {self.enc} encounter checks",
                "npl": c["npl"], "ntp": c["ntp"], "dt": c["dt"], "rhscale": c["rhscale"], "seed": c["seed"],
                "precision": precision, "l2": "flushed before every timed step (512 MB memset, untimed)"}

    def oracle_sample(self, budget_s):
        from oracle import oracle as O
        c = self.cfg
        s = O.OracleSystem("SYMBA", self.cb, self.pl, self.tp, dt=c["dt"], rhscale=c["rhscale"], lclose=True,
                           encounter_check_plpl=self.enc, encounter_check_pltp=self.enc)
        s.step(1)
        n, t0 = 0, time.perf_counter()
        while True:
            s.step(1)
            n += 1
            el = time.perf_counter() - t0
            if el > budget_s or n >= 200:
                break
        return self.nbodies * n, el, f"{n} SyMBA steps of the C1 system ({self.nbodies} bodies) after 1 warm-up step"


# ---------------------------------------------------------------- measurement
class ClockSampler:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.i0 = self.i1 = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()  # the timed region starts once sampling runs
            while not self.rows and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.i0 = len(self.rows)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        self.i1 = len(self.rows)
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
        rows = self.rows[self.i0:self.i1] or self.rows[max(0, self.i0 - 1):self.i0 + 1]  # in the timed region
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "samples_in_timed_region": self.i1 - self.i0}


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def rel_energy(e0, e1):
    """Relative energy and angular-momentum errors between two energy snapshots, as arrays over
    systems (one entry for a single system), with the reference's collision bookkeeping
    (swiftest_io.f90:153,181-183): the energy the collision resolutions changed (E_collisions)
    is taken out of dE, and dL_ref adds the angular momentum booked as escaped (L_escape).
    dE uses the central-body potential at the heliocentric distance, dE_ref the reference's
    own formula (barycentric distance)."""
    def arr(x):
        return np.atleast_1d(np.asarray(x, dtype=np.float64))
    Ec = arr(e1.get("E_collisions", 0.0)) - arr(e0.get("E_collisions", 0.0))
    dE = np.abs(arr(e1["te_helio"]) - arr(e0["te_helio"]) - Ec) / np.abs(arr(e0["te_helio"]))
    dEr = np.abs(arr(e1["te"]) - arr(e0["te"]) - Ec) / np.abs(arr(e0["te"]))
    L0, L1 = np.atleast_2d(e0["L"]), np.atleast_2d(e1["L"])
    esc = np.atleast_2d(e1.get("L_escape", np.zeros(3))) - np.atleast_2d(e0.get("L_escape", np.zeros(3)))
    dL = np.linalg.norm(L1 - L0, axis=1) / np.linalg.norm(L0, axis=1)
    dLr = np.linalg.norm(L1 + esc - L0, axis=1) / np.linalg.norm(L0, axis=1)
    return dE, dEr, dL, dLr


def err_summary(dE, dEr, dL, dLr):
    return {"dE_E_max": float(dE.max()), "dE_E_median": float(np.median(dE)), "dE_E_ref_formula_max": float(dEr.max()),
            "dL_L_max": float(dL.max()), "dL_L_ref_formula_max": float(dLr.max())}


def run_path(ctx, wl, precision, steps, warmup, prof_steps=0, clocks=None):
    """W warm-up steps, K timed steps, then prof_steps steps under the per-class CUDA-event
    profile (which serialises the step: the closing kick of systems without encounters
    no longer overlaps the recursion), all from the same initial conditions."""
    s = wl.make(ctx, precision)
    e0 = s.energy()
    s.step(warmup)
    ctx.synchronize()
    launches0 = ctx.launches
    total_ms = 0.0
    with clocks if clocks is not None else _Null():
        for _ in range(steps):
            ctx.flush_l2()
            ctx.event_record(0)
            s.step(1)
            ctx.event_record(1)
            total_ms += ctx.event_elapsed_ms(0, 1)
    launches = ctx.launches - launches0  # kernels of ours (the L2-flush memsets are not counted)
    prof, prof_ms = None, 0.0
    if prof_steps:
        s.profile(True)
        for _ in range(prof_steps):
            ctx.flush_l2()
            ctx.event_record(0)
            s.step(1)
            ctx.event_record(1)
            prof_ms += ctx.event_elapsed_ms(0, 1)
        prof = s.profile_read()
        s.profile(False)
    e1 = s.energy()
    stats = s.stats()
    plan = None
    if hasattr(s, "kick_strip") and precision == "MIXED":  # ensembles: the autotuned mixed kicks
        kv = s.kick_variant()
        plan = {"plpl": "symmetric" if kv["pl"] == 5 else f"broadcast shape {kv['pl']}",
                "plpl_tile": s.kick_tile(), "plpl_strip": s.kick_strip(), "plpl_warps_per_block": s.kick_warps(),
                "plpl_row_group": s.kick_group(),
                "pltp_shape": kv["tp"]}
    s.close()
    return total_ms, launches, (prof, prof_ms), rel_energy(e0, e1), stats, plan


def run_e2e(ctx, wl, precision, steps):
    """The same metric through the public API with host buffers: every step uploads the
    state (pinned host arrays -> device), steps once and reads the state back.  Returns the
    time and the bytes of the state arrays, which every step copies in each direction."""
    import torch
    s = wl.make(ctx, precision)
    s.step(2)
    pinned = [torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy() for shape in wl.state_arrays()]
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


def cpu_baseline(wl, budget_s):
    """The oracle (C restatement of the reference's OpenMP path) on this host, on a bounded
    sample of the same workload."""
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    from oracle import oracle as O
    O.build()
    bs, el, sample = wl.oracle_sample(budget_s)
    return {"value": bs / el, "unit": UNIT, "cores": int(os.environ.get("OMP_NUM_THREADS", threads)), "kind": "port",
            "sample": f"{sample}, {el:.1f} s, C restatement of the reference loops with OpenMP"}


def reference_arm(args, world, rank):
    if rank != 0:
        return 0
    wl = {"c4": C4, "c3": C3, "c3w": C3W, "c1": C1}[args.workload](args)
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    from oracle import oracle as O
    O.build()
    budget = max(0.5, min(6.0, 150.0 / max(1, args.steps + args.warmup)))  # whole run ~2.5 min
    for _ in range(args.warmup):
        wl.oracle_sample(budget / 4)
    bs_tot, el_tot, sample = 0, 0.0, ""
    for _ in range(args.steps):
        bs, el, sample = wl.oracle_sample(budget)
        bs_tot += bs
        el_tot += el
    v = bs_tot / el_tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el_tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, numpy default_rng)",
            "config": wl.config("FP64 CPU"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                             "sample": f"each step: {sample} (C restatement of the reference's OpenMP loops; the "
                                       "Fortran reference cannot be compiled on this image)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def load_traffic(key, plan=None):
    """DRAM bytes per launch of a kernel class from the ncu capture recorded in
    profiles/traffic.json (bytes, the capture's command, the commit it ran and the kick shape
    it captured), or None when there is none or it captured another shape than `plan` (the
    kick shape this run used)."""
    p = ROOT / "profiles" / "traffic.json"
    try:
        rec = json.loads(p.read_text()).get(key)
    except (OSError, json.JSONDecodeError):
        return None, None
    if not isinstance(rec, dict):
        return None, None
    src = {k: rec.get(k) for k in ("commit", "command", "note", "plan")}
    shape = rec.get("plan")
    if plan and isinstance(shape, dict) and any(plan.get(k) != v for k, v in shape.items()):
        src["note"] = "not used: the recorded capture is of another kick shape than this run's " + json.dumps(
            {k: plan.get(k) for k in shape})
        return None, src
    return rec.get("bytes_per_launch"), src


def main():
    args = parse()
    world, rank, local, td = dist_setup(args)
    if args.impl == "reference":
        return reference_arm(args, world, rank)
    from swiftest_gb300 import build as B
    B.build()
    from swiftest_gb300.api import Context
    wl = {"c4": C4, "c3": C3, "c3w": C3W, "c1": C1}[args.workload](args)
    ctx = Context(local)
    clocks = ClockSampler(local)
    if td:
        td.barrier()
    nprof = max(3, min(10, args.steps))
    ms_mixed, launches, (prof, prof_ms), err_m, st_m, plan = run_path(ctx, wl, "MIXED", args.steps, args.warmup,
                                                                      nprof, clocks=clocks)
    steps64 = args.steps  # same steps as the mixed arm, so the two |dE/E| are over the same run
    ms_fp64, _, (prof64, _), err_f, st_f, _ = run_path(ctx, wl, "FP64", steps64, args.warmup, nprof)
    e2e_ms, e2e_bytes = run_e2e(ctx, wl, "MIXED", args.steps)
    ms_mixed, ms_fp64, e2e_ms = max_over_ranks(td, [ms_mixed, ms_fp64, e2e_ms])
    nb = wl.nbodies
    value = whole_job_rate(world, nb, args.steps, ms_mixed)
    fp64_value = whole_job_rate(world, nb, steps64, ms_fp64)

    # roofline of the pair kick (mixed path), from the live CUDA-event profile on the library's stream
    peak32_scalar = ctx.probe_peak_tflops("fp32")
    peak32_packed = ctx.probe_peak_tflops("fp32x2")
    peak32 = max(peak32_scalar, peak32_packed)  # the kick issues packed f32x2 FMAs: the larger rate bounds it
    peak64 = ctx.probe_peak_tflops("fp64")
    traffic, traffic_src = load_traffic(f"kick_pl_{args.workload}", plan)
    roof = None
    kick = prof["kick_pl"]
    if kick["launches"]:
        avg_ms = kick["ms"] / kick["launches"]
        flops = FLOPS_PER_INTERACTION * wl.plpl_pairs  # one pl-pl evaluation
        ach = flops / (avg_ms * 1e-3) / 1e12
        roof = {"kernel": "kick_pl (mixed FP32 pair kick, batched persistent launch)", "bound": "fp32",
                "achieved": ach, "peak": peak32, "unit": "TFLOP/s", "frac": ach / peak32 if peak32 else None,
                "peak_source": "larger of the FP32 FMA-chain probes measured by bench.py on this GPU, scalar "
                               f"FFMA {peak32_scalar:.1f} and packed f32x2 FMA {peak32_packed:.1f} TFLOP/s "
                               "(MEASURED_PEAKS.json has no FP32 figure)",
                "algorithmic_flops_per_launch": flops, "avg_launch_ms": avg_ms,
                "traffic": traffic, "traffic_source": traffic_src}
    kernel_profile = {"steps": nprof, "ms_per_step": prof_ms / nprof,
                      **{k: {"launches": v["launches"], "ms_total": round(v["ms"], 4),
                             "share": round(v["ms"] / prof_ms, 4)} for k, v in prof.items()}}
    dom = max(prof, key=lambda k: prof[k]["ms"])  # of the profiled (serialised) steps
    cpu = cpu_baseline(wl, args.cpu_seconds) if rank == 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_mixed / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (f32 pair kicks)", "data": "synthetic (seeded, numpy default_rng)",
        "config": wl.config("mixed"),
        "fp64_path": {"value": fp64_value, "steps": steps64, "ms_per_step": ms_fp64 / steps64, **err_summary(*err_f),
                      "stats": st_f,
                      "kernel_profile": {k: {"launches": v["launches"], "ms_total": round(v["ms"], 4)}
                                         for k, v in prof64.items()}},
        "mixed_path": {**err_summary(*err_m), "stats": st_m, "kick_plan": plan},
        "speedup_mixed_vs_fp64": value / fp64_value,
        "pair_interactions_per_s": whole_job_rate(world, wl.pairs_per_step, args.steps, ms_mixed),
        "kernel_profile": kernel_profile, "dominant_kernel_class": dom,
        "roofline": roof, "fp64_peak_probe_tflops": peak64,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "e2e": {"value": whole_job_rate(world, nb, args.steps, e2e_ms), "unit": UNIT,
                "h2d_bytes_per_step": e2e_bytes, "d2h_bytes_per_step": e2e_bytes},
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
