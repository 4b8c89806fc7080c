"""Run one hot-path kernel on a C1-shaped workload, for profilers (ncu) and quick timing.

    python benchmarks/profile_cases.py <case> [--npl N] [--ntp M] [--reps R]

cases: kick_tp_mixed, kick_pl_mixed, kick_tp_fp64, kick_pl_fp64, drift, encounter_pltp,
encounter_plpl (and _sas: sort-and-sweep), symba_mixed, symba_fp64 (inputs: the seeded C1 disk, AU, Msun, yr), and
ens_mixed, ens_fp64 (steps of a batched ensemble, first --nsys systems: --ensemble C4, the
SyMBA disks, or C3 / C3W, the HELIO / WHM systems with 5 tp per pl).
Prints the average wall time per call (host buffers, so it includes the copies).
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("case")
    p.add_argument("--npl", type=int, default=2000)
    p.add_argument("--ntp", type=int, default=10000)
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--nsys", type=int, default=None)
    p.add_argument("--ensemble", default="C4", choices=["C4", "C3", "C3W"])
    p.add_argument("--encounter", default="TRIANGULAR", choices=["TRIANGULAR", "SORTSWEEP"],
                   help="level-0 check mode of the SyMBA cases")
    for k, h in (("tile", "bodies per tile"), ("strip", "tiles J per item"), ("warps", "warps per block"),
                 ("group", "tiles per row group")):
        p.add_argument(f"--kick-{k}", type=int, default=0,
                       help=f"ens_mixed: the symmetric pl-pl kick's {h} (0: autotuned; forcing all four skips "
                            "the tuner's timing launches)")
    a = p.parse_args(argv)
    from swiftest_gb300 import SWG_ENC_SORTSWEEP, SWG_FP64, SWG_MIXED
    from swiftest_gb300 import build as B
    from swiftest_gb300 import initial_conditions as IC
    from swiftest_gb300.api import Context, NBodySystem
    B.build()
    cb, pl, tp = IC.make_system(seed=0, npl=a.npl, ntp=a.ntp, amin=0.3, amax=3.0)
    pl = IC.sort_for_integrator(pl, "SYMBA")
    ctx = Context(0)
    renc = pl["rhill"]
    cases = {
        "kick_tp_mixed": lambda: ctx.kick_getacch_int_all_tp(tp["rh"], pl["rh"], pl["Gmass"], precision=SWG_MIXED),
        "kick_pl_mixed": lambda: ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"],
                                                                 precision=SWG_MIXED),
        "kick_tp_fp64": lambda: ctx.kick_getacch_int_all_tp(tp["rh"], pl["rh"], pl["Gmass"], precision=SWG_FP64),
        "kick_pl_fp64": lambda: ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"],
                                                                precision=SWG_FP64),
        "drift": lambda: ctx.drift_all(IC.GMCB, tp["rh"], tp["vh"], 0.005),
        "encounter_pltp": lambda: ctx.encounter_check_all_pltp(pl["rh"], pl["vh"], tp["rh"], tp["vh"], renc, 0.005),
        "encounter_plpl": lambda: ctx.encounter_check_all_plpl(pl["rh"], pl["vh"], renc, 0.005),
        "encounter_pltp_sas": lambda: ctx.encounter_check_all_pltp(pl["rh"], pl["vh"], tp["rh"], tp["vh"], renc, 0.005,
                                                                   mode=SWG_ENC_SORTSWEEP),
        "encounter_plpl_sas": lambda: ctx.encounter_check_all_plpl(pl["rh"], pl["vh"], renc, 0.005,
                                                                   mode=SWG_ENC_SORTSWEEP),
    }
    enc = {} if a.encounter == "TRIANGULAR" else dict(encounter_check_plpl=a.encounter,
                                                      encounter_check_pltp=a.encounter)
    if a.case.startswith("ens"):
        from swiftest_gb300.api import Ensemble
        if a.ensemble == "C3W":
            E = IC.make_ensemble("C3", nsys=a.nsys, integrator="WHM")
        else:
            E = IC.make_ensemble(a.ensemble, nsys=a.nsys)
        ens = Ensemble(ctx, E, precision="MIXED" if a.case.endswith("mixed") else "FP64",
                       **(enc if E["integrator"] == "SYMBA" else {}))
        ens.set_kick_tile(a.kick_tile)
        ens.set_kick_strip(a.kick_strip)
        ens.set_kick_warps(a.kick_warps)
        ens.set_kick_group(a.kick_group)
        run = lambda: ens.step(1)  # noqa: E731
    elif a.case.startswith("symba"):
        prec = "MIXED" if a.case.endswith("mixed") else "FP64"
        s = NBodySystem(ctx, "SYMBA", cb, pl, tp, dt=0.005, rhscale=1.0, precision=prec, **enc)
        run = lambda: s.step(1)  # noqa: E731
    else:
        run = cases[a.case]
    run()
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.reps):
        run()
    ctx.synchronize()
    print(f"{a.case}: {1e3 * (time.perf_counter() - t0) / a.reps:.3f} ms per call (host buffers)")
    ctx.close()


if __name__ == "__main__":
    main()
