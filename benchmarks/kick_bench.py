"""Standalone pair-kick benchmark (large single systems) through the C ABI with device pointers.

    python benchmarks/kick_bench.py [--n 16384 65536 131072] [--reps 3]

For each N: N massive bodies (masses log-uniform in [1e-12, 1e-8] Msun, a in [0.5, 5] AU,
seed 0) and 4N test particles; one evaluation of
  * the triangular pl-pl kick (swiftest_kick_getacch_int_all_tri_*),
  * the flat pl-pl kick over the canonical pair list (swiftest_kick_getacch_int_all_flat_*),
  * the pl-tp kick (swiftest_kick_getacch_int_all_tp),
in FP64 (reference operation order) and in mixed precision, timed with CUDA events on the
library's stream (inputs resident on the device, best of --reps).  Reported per N and path:
ordered pair interactions per second, the equivalent TFLOP/s at 20 flop per interaction
and its fraction of the measured FMA-chain peak (FP64 or FP32), and the mixed path's
max / RMS relative acceleration error against the FP64 path (which the parity tests
show bit-identical to the oracle).  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

FLOPS_PER_INTERACTION = 20.0


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, nargs="+", default=[16384, 65536, 131072])
    p.add_argument("--reps", type=int, default=3)
    a = p.parse_args(argv)
    import torch

    from swiftest_gb300 import _lib as L
    from swiftest_gb300 import build as B
    from swiftest_gb300 import initial_conditions as IC
    from swiftest_gb300.api import Context
    B.build()
    ctx = Context(0)
    lib = ctx.lib
    peak = {L.SWG_FP64: ctx.probe_peak_tflops("fp64"), L.SWG_MIXED: ctx.probe_peak_tflops("fp32")}
    out = {"peaks_tflops": {"fp64": peak[L.SWG_FP64], "fp32": peak[L.SWG_MIXED]}, "results": []}
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for N in a.n:
        _, pl, tp = IC.make_system(seed=0, npl=N, ntp=4 * N, mmin=1e-12, mmax=1e-8, amin=0.5, amax=5.0)
        r, g, R = _dev(torch, pl["rh"], np.float64), _dev(torch, pl["Gmass"], np.float64), \
            _dev(torch, pl["radius"], np.float64)
        rt = _dev(torch, tp["rh"], np.float64)
        mask = torch.ones(4 * N, dtype=torch.int32, device="cuda")
        acc = torch.zeros((N, 3), dtype=torch.float64, device="cuda")
        acct = torch.zeros((4 * N, 3), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        npairs = N * (N - 1) // 2

        def call(kind, prec):  # acc accumulates, as in the reference
            if kind == "tri":
                rc = lib.swg_kick_getacch_int_all_tri_pl(ctx.h, N, N, vp(r), vp(g), vp(R), vp(acc), prec,
                                                         L.SWG_MEM_DEVICE)
            elif kind == "flat":
                rc = lib.swg_kick_getacch_int_all_flat_pl(ctx.h, N, N, npairs, None, vp(r), vp(g), vp(R), vp(acc),
                                                          prec, L.SWG_MEM_DEVICE)
            else:
                rc = lib.swg_kick_getacch_int_all_tp(ctx.h, 4 * N, N, vp(rt), vp(r), vp(g), vp(mask), vp(acct),
                                                     prec, L.SWG_MEM_DEVICE)
            ctx.check("kick", rc)

        res = {"n_pl": N, "n_tp": 4 * N}
        keep = {}
        for kind in ("tri", "flat", "tp"):
            inter = N * (N - 1) if kind != "tp" else 4 * N * N
            for prec, name in ((L.SWG_FP64, "fp64"), (L.SWG_MIXED, "mixed")):
                acc.zero_()
                acct.zero_()
                torch.cuda.synchronize()
                call(kind, prec)  # one evaluation from zero: the accuracy snapshot
                ctx.synchronize()
                keep[(kind, name)] = (acct if kind == "tp" else acc).cpu().numpy().copy()
                best = None
                for _ in range(a.reps):
                    ctx.flush_l2()
                    ctx.event_record(0)
                    call(kind, prec)
                    ctx.event_record(1)
                    ms = ctx.event_elapsed_ms(0, 1)
                    best = ms if best is None else min(best, ms)
                ctx.synchronize()
                tfl = FLOPS_PER_INTERACTION * inter / (best * 1e-3) / 1e12
                res[f"{kind}_{name}"] = {"ms": best, "interactions_per_s": inter / (best * 1e-3), "tflops": tfl,
                                         "frac_of_peak": tfl / peak[prec]}
            f, m = keep[(kind, "fp64")], keep[(kind, "mixed")]
            rel = np.linalg.norm(m - f, axis=1) / np.linalg.norm(f, axis=1)
            res[f"{kind}_mixed"]["rel_err_max"] = float(rel.max())
            res[f"{kind}_mixed"]["rel_err_rms"] = float(np.sqrt(np.mean(rel ** 2)))
        out["results"].append(res)
        del r, g, R, rt, mask, acc, acct
        torch.cuda.empty_cache()
    print(json.dumps(out), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
