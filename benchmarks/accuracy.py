"""Long-run accuracy of the mixed-precision batched path against the FP64 path, C4 ensemble.

    python benchmarks/accuracy.py [--steps S] [--every K] [--sample N] [--nsys M] [--out FILE]

1. The whole C4 ensemble (256 planetesimal disks, SyMBA, dt = 0.002 yr, 1-Hill-radius
   encounter radius) runs S steps in mixed precision.  Recorded per system: |dE/E| with the
   collision energy taken out as the reference's error terms do (central-body potential at
   the heliocentric distance; the reference's own formula is recorded too), |dL/L| of the
   system's angular momentum, the number of merges (bodies left INACTIVE), and the history of
   |dE/E| every K steps.
2. The FP64 path (the reference's operation order) then runs the same S steps on a subset of
   the systems, batched together (each system's FP64 trajectory is independent of the others
   in the batch): a random sample of N systems without merges (numpy default_rng(2024)), then
   every system with a merge and every system whose mixed |dE/E| exceeds twice the largest
   FP64 error of the sample.
3. One JSON line: per-system tables, the mixed / FP64 ratio per compared system and its
   maximum, and the wall times.

--nsys M takes the first M systems instead of all 256 (quick runs).

--twin S runs system S in FP64 several times, batched: as generated and with its first
body's x moved by each relative amount of --perturb (one unit in the last place when 0); the
|dE/E| of the copies show how the FP64 error of that system depends on a perturbation of the
size the mixed path's FP32 pair arithmetic makes (~1e-7 relative in each pair force).

--fp64-from FILE reuses the FP64 errors of a recorded run (the per-system table of
profiles/accuracy_c4_10k_steps.md) instead of rerunning the FP64 sample: the FP64 path is the
reference's operation order, bit-identical to the oracle, so its trajectories do not change
with the mixed path's kernels.  The FP64 path then runs only the systems outside that table
that merge in this mixed run or exceed --outlier-threshold.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def _errors(e0, e1):
    """|dE/E| (heliocentric central-body potential; and the reference's formula) and |dL/L|
    per system, with the collision bookkeeping taken out as bench.rel_energy does."""
    from bench import rel_energy
    dE, dEr, dL, _ = rel_energy(e0, e1)
    return dE, dEr, dL


def subset(E, idx):
    """The systems idx of a packed ensemble E, packed again."""
    systems = [E["systems"][i] for i in idx]
    out = {k: E[k] for k in ("integrator", "dt", "rhscale")}
    out["npl"] = E["npl"][idx].copy()
    out["ntp"] = E["ntp"][idx].copy()
    out["GMcb"] = np.asarray(E["GMcb"])[idx].copy()
    out["Rcb"] = np.asarray(E["Rcb"])[idx].copy()
    out["pl"] = {k: np.concatenate([p[k] for p, _ in systems]) for k in ("rh", "vh", "Gmass", "radius", "rhill")}
    ntp = sum(len(t["rh"]) for _, t in systems)
    out["tp"] = {k: (np.concatenate([t[k] for _, t in systems]) if ntp else np.zeros((0, 3))) for k in ("rh", "vh")}
    out["systems"] = systems
    return out


def run(ctx, E, precision, steps, every):
    from swiftest_gb300.api import Ensemble
    ens = Ensemble(ctx, E, precision=precision)
    e0 = ens.energy()
    hist = []
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        k = min(every, steps - done)
        ens.step(k)
        done += k
        dE, _, _ = _errors(e0, ens.energy())
        hist.append(dE.tolist())
    wall = time.perf_counter() - t0
    e1 = ens.energy()
    dE, dEr, dL = _errors(e0, e1)
    _, _, st = ens.get_pl()
    merges = [int((st[ens.poff[s]:ens.poff[s + 1]] == 1).sum()) for s in range(len(E["npl"]))]
    stats = ens.stats()
    ens.close()
    return {"dE_E": dE.tolist(), "dE_E_ref_formula": dEr.tolist(), "dL_L": dL.tolist(), "merges": merges,
            "E_collisions_over_E0": (np.abs(e1["E_collisions"]) / np.abs(e0["te"])).tolist(),
            "history_every": every, "history": hist, "stats": stats, "wall_s": wall}


def recorded_fp64(path):
    """{system: {dE_E, dL_L, merges}} of the FP64 path from a recorded table (rows
    system | N_pl | why | merges mixed / FP64 | FP64 dE | mixed dE | ratio | FP64 dL | mixed dL)."""
    out = {}
    for line in Path(path).read_text().splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) != 9 or not cells[0].isdigit():
            continue
        out[int(cells[0])] = {"dE_E": float(cells[4]), "dL_L": float(cells[7]),
                              "merges": int(cells[3].split("/")[1]), "why": cells[2]}
    return out


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--steps", type=int, default=10000)
    p.add_argument("--every", type=int, default=1000)
    p.add_argument("--sample", type=int, default=32)
    p.add_argument("--nsys", type=int, default=None)
    p.add_argument("--out", default=None)
    p.add_argument("--fp64-from", default=None, help="recorded FP64 per-system table to reuse")
    p.add_argument("--twin", type=int, default=None, help="FP64 runs of one system and perturbed copies")
    p.add_argument("--perturb", default="0", help="--twin: relative moves of the first body's x (0: one ulp)")
    p.add_argument("--outlier-threshold", type=float, default=None,
                   help="with --fp64-from: mixed |dE/E| above which a system outside the table runs in FP64")
    a = p.parse_args(argv)
    from swiftest_gb300 import build as B
    from swiftest_gb300 import initial_conditions as IC
    from swiftest_gb300.api import Context
    B.build()
    ctx = Context(0)
    E = IC.make_ensemble("C4", nsys=a.nsys)
    nsys = len(E["npl"])
    if a.twin is not None:
        return twin(a, ctx, E)
    out = {"workload": f"C4 ensemble, {nsys} systems ({int(E['npl'].sum())} pl), SyMBA, dt=0.002 yr, RHSCALE=1.0, "
                       f"{a.steps} steps", "steps": a.steps, "npl": E["npl"].tolist()}
    mixed = run(ctx, E, "MIXED", a.steps, a.every)
    out["mixed"] = mixed
    dEm = np.array(mixed["dE_E"])
    merged = [s for s in range(nsys) if mixed["merges"][s] > 0]
    if a.fp64_from:
        return compare_recorded(a, ctx, E, out, mixed, dEm, merged)
    rng = np.random.default_rng(2024)
    rest = [s for s in range(nsys) if s not in merged]
    sample = sorted(int(x) for x in rng.choice(rest, size=min(a.sample, len(rest)), replace=False))
    # the FP64 sample first: its largest error sets the outlier threshold for the mixed path
    fp_sample = run(ctx, subset(E, np.array(sample)), "FP64", a.steps, a.every)
    thresh = 2.0 * max(fp_sample["dE_E"])
    outliers = [s for s in range(nsys) if dEm[s] > thresh and s not in merged and s not in sample]
    extra = sorted(set(merged) | set(outliers))
    fp_extra = run(ctx, subset(E, np.array(extra)), "FP64", a.steps, a.every) if extra else None
    keys = ("dE_E", "dE_E_ref_formula", "dL_L", "merges")
    fp = {s: {key: fp_sample[key][k] for key in keys} for k, s in enumerate(sample)}
    if fp_extra:
        fp.update({s: {key: fp_extra[key][k] for key in keys} for k, s in enumerate(extra)})
    rows = []
    for s in sorted(fp):
        rows.append({"system": s, "npl": int(E["npl"][s]),
                     "why": "merge" if s in merged else ("outlier" if s in outliers else "sample"),
                     "merges_mixed": mixed["merges"][s], "merges_fp64": fp[s]["merges"],
                     "dE_E_fp64": fp[s]["dE_E"], "dE_E_mixed": float(dEm[s]),
                     "ratio": float(dEm[s] / max(fp[s]["dE_E"], 1e-300)),
                     "dL_L_fp64": fp[s]["dL_L"], "dL_L_mixed": mixed["dL_L"][s]})
    out["compared"] = rows
    out["outlier_threshold"] = thresh
    out["ratio_max"] = max(r["ratio"] for r in rows)
    out["fp64_wall_s"] = fp_sample["wall_s"] + (fp_extra["wall_s"] if fp_extra else 0.0)
    out["fp64_max_over_compared"] = max(r["dE_E_fp64"] for r in rows)
    out["mixed_max_over_compared"] = max(r["dE_E_mixed"] for r in rows)
    out["mixed_max_all"] = float(dEm.max())
    line = json.dumps(out)
    if a.out:
        Path(a.out).write_text(line + "\n")
    print(json.dumps({k: out[k] for k in ("workload", "ratio_max", "mixed_max_all", "fp64_max_over_compared",
                                          "mixed_max_over_compared", "fp64_wall_s")}), flush=True)
    ctx.close()


def twin(a, ctx, E):
    """FP64 runs of system a.twin and of copies whose first body's x is moved."""
    moves = [float(x) for x in a.perturb.split(",")]
    one = subset(E, np.array([a.twin] * (1 + len(moves))))
    n = int(one["npl"][0])
    pl = {k: v.copy() for k, v in one["pl"].items()}
    for c, m in enumerate(moves, start=1):
        x = pl["rh"][c * n, 0]
        pl["rh"][c * n, 0] = np.nextafter(x, np.inf) if m == 0 else x * (1.0 + m)
    one["pl"] = pl
    res = run(ctx, one, "FP64", a.steps, a.every)
    out = {"system": a.twin, "npl": n, "steps": a.steps, "perturb": [None] + moves, "dE_E": res["dE_E"],
           "merges": res["merges"], "history": res["history"],
           "ratios": [d / max(res["dE_E"][0], 1e-300) for d in res["dE_E"]], "wall_s": res["wall_s"]}
    if a.out:
        Path(a.out).write_text(json.dumps(out) + "\n")
    print(json.dumps(out), flush=True)
    ctx.close()
    return 0


def compare_recorded(a, ctx, E, out, mixed, dEm, merged):
    """The mixed run against recorded FP64 errors, plus FP64 runs of the systems the record
    lacks (new merges, or mixed errors above the threshold)."""
    rec = recorded_fp64(a.fp64_from)
    nsys = len(E["npl"])
    thresh = a.outlier_threshold if a.outlier_threshold is not None else 2.0 * max(
        v["dE_E"] for v in rec.values() if v["why"] == "sample")
    outliers = [s for s in range(nsys) if dEm[s] > thresh and s not in merged]
    extra = sorted(s for s in set(merged) | set(outliers) if s not in rec)
    fp_extra = run(ctx, subset(E, np.array(extra)), "FP64", a.steps, a.every) if extra else None
    fp = {s: dict(v, source="recorded") for s, v in rec.items() if s < nsys}
    if fp_extra:
        fp.update({s: {"dE_E": fp_extra["dE_E"][k], "dL_L": fp_extra["dL_L"][k], "merges": fp_extra["merges"][k],
                       "source": "run"} for k, s in enumerate(extra)})
    rows = []
    for s in sorted(fp):
        rows.append({"system": s, "npl": int(E["npl"][s]),
                     "why": "merge" if s in merged else ("outlier" if s in outliers else fp[s].get("why", "sample")),
                     "fp64": fp[s]["source"], "merges_mixed": mixed["merges"][s], "merges_fp64": fp[s]["merges"],
                     "dE_E_fp64": fp[s]["dE_E"], "dE_E_mixed": float(dEm[s]),
                     "ratio": float(dEm[s] / max(fp[s]["dE_E"], 1e-300)),
                     "dL_L_fp64": fp[s]["dL_L"], "dL_L_mixed": mixed["dL_L"][s]})
    out["compared"] = rows
    out["outlier_threshold"] = thresh
    out["ratio_max"] = max(r["ratio"] for r in rows)
    out["fp64_wall_s"] = fp_extra["wall_s"] if fp_extra else 0.0
    out["fp64_run_systems"] = extra
    out["mixed_max_all"] = float(dEm.max())
    out["mixed_median_all"] = float(np.median(dEm))
    line = json.dumps(out)
    if a.out:
        Path(a.out).write_text(line + "\n")
    print(json.dumps({k: out[k] for k in ("workload", "ratio_max", "mixed_max_all", "mixed_median_all",
                                          "fp64_run_systems", "fp64_wall_s")}), flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    main()
