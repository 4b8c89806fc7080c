"""Long-run accuracy of the mixed-precision batched path against the FP64 path.

    python benchmarks/accuracy.py [--nsys N] [--steps S] [--every K] [--full-mixed]

Steps the first N systems of the C4 ensemble (256 planetesimal disks, SyMBA, dt = 0.002 yr,
1-Hill-radius encounter radius) for S steps in both precisions from the same initial
conditions and prints one JSON line: per-system |dE/E| (central-body potential at the
heliocentric distance, and the reference's formula) and |dL/L| at the end, their
maxima and medians per path, the ratio of the mixed to the FP64 error, and the number of
steps with encounters.  With --full-mixed the whole 256-system ensemble is also run in
mixed precision (the FP64 path at that size takes ~0.27 s per step).
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


def _run(ctx, E, precision, steps, every):
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
        hist.append([done, float(dE.max()), float(np.median(dE))])
    wall = time.perf_counter() - t0
    dE, dEr, dL = _errors(e0, ens.energy())
    st = ens.stats()
    ens.close()
    return {"dE_E": dE.tolist(), "dE_E_ref_formula": dEr.tolist(), "dL_L": dL.tolist(),
            "dE_E_max": float(dE.max()), "dE_E_median": float(np.median(dE)), "dL_L_max": float(dL.max()),
            "history": hist, "stats": st, "wall_s": wall}


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--nsys", type=int, default=16)
    p.add_argument("--steps", type=int, default=10000)
    p.add_argument("--every", type=int, default=1000)
    p.add_argument("--full-mixed", action="store_true")
    a = p.parse_args(argv)
    from swiftest_gb300 import build as B
    from swiftest_gb300 import initial_conditions as IC
    from swiftest_gb300.api import Context
    B.build()
    ctx = Context(0)
    E = IC.make_ensemble("C4", nsys=a.nsys)
    out = {"workload": f"first {a.nsys} systems of the C4 ensemble ({int(E['npl'].sum())} pl), SyMBA, dt=0.002 yr, "
                       f"RHSCALE=1.0, {a.steps} steps", "steps": a.steps}
    out["fp64"] = _run(ctx, E, "FP64", a.steps, a.every)
    out["mixed"] = _run(ctx, E, "MIXED", a.steps, a.every)
    f, m = np.array(out["fp64"]["dE_E"]), np.array(out["mixed"]["dE_E"])
    out["ratio_mixed_over_fp64_max"] = float(m.max() / f.max())
    out["ratio_mixed_over_fp64_per_system_max"] = float(np.max(m / np.maximum(f, 1e-300)))
    if a.full_mixed:
        Efull = IC.make_ensemble("C4")
        r = _run(ctx, Efull, "MIXED", a.steps, a.every)
        out["full_c4_mixed"] = {k: r[k] for k in ("dE_E_max", "dE_E_median", "dL_L_max", "history", "stats",
                                                   "wall_s")}
    print(json.dumps(out), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
