"""Timeline of one SyMBA step on the GPU: when each stream finishes each phase.

    python benchmarks/step_timeline.py [--workload c4|c1] [--steps 30] [--show 3]

Builds a copy of the library (under _build/) whose step loops (ensemble.cu ens_step for the
C4 ensemble, system.cu symba_step / symba_interp for the C1 disk) record a timed CUDA event
after each phase on the stream that ran it, and the host clock when the host enqueued it.
It then steps the seeded workload with the mixed path and prints, for the last --show steps,
each mark's GPU completion time and host enqueue time relative to the step's first mark
(microseconds), and the averages over all steps after the first --skip.  The marks only
record events between the phases; the phases' work and streams are unchanged.  Measurement
tool: the product library is not touched.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import shutil
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

TRACE_DEF = r"""
#include <chrono>
#include <vector>
namespace swg_trace {
struct Rec { int id; cudaEvent_t ev; double host_us; };
std::vector<Rec> recs;
bool on = false;
}
void swg_tr(cudaStream_t st, int id) {
    if (!swg_trace::on) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, st);
    const double h = std::chrono::duration<double, std::micro>(
        std::chrono::steady_clock::now().time_since_epoch()).count();
    swg_trace::recs.push_back({id, e, h});
}
extern "C" int swg_trace_enable(int on) { swg_trace::on = on != 0; return 0; }
// ids, GPU ms after the first record, host us after the first record; returns the count
extern "C" int swg_trace_read(int cap, int *ids, float *gpu_ms, double *host_us) {
    cudaDeviceSynchronize();
    const int n = (int)swg_trace::recs.size();
    for (int k = 0; k < n && k < cap; k++) {
        ids[k] = swg_trace::recs[k].id;
        cudaEventElapsedTime(&gpu_ms[k], swg_trace::recs[0].ev, swg_trace::recs[k].ev);
        host_us[k] = swg_trace::recs[k].host_us - swg_trace::recs[0].host_us;
    }
    for (auto &r : swg_trace::recs) cudaEventDestroy(r.ev);
    swg_trace::recs.clear();
    return n;
}
"""

# mark ids: (name, stream)
MARKS = {
    0: ("step start", "main"),
    1: ("level-0 checks queued/done", "side"),
    2: ("opening sums", "main"),
    3: ("opening pair accelerations", "main"),
    4: ("lists finalized", "side"),
    5: ("opening kick applied", "main"),
    6: ("item flags", "main"),
    7: ("recursion kernel", "main"),
    8: ("level-0 drift", "side"),
    9: ("unlisted closing items + sums", "side"),
    10: ("recursion finished (pauses resolved)", "main"),
    11: ("listed closing items", "main"),
    12: ("closing sums joined", "main"),
    13: ("closing kick, linear drift, vb2vh", "main"),
    14: ("step end", "main"),
    20: ("step start", "main"),
    21: ("level-0 lists joined (opening sums + pl accelerations beside them)", "main"),
    22: ("opening pl kick applied", "main"),
    23: ("pl drift", "main"),
    24: ("tp opening half-step", "side"),
    25: ("recursion", "main"),
    26: ("closing pl kick", "main"),
    27: ("tp closing kick", "side"),
    28: ("step end", "main"),
}


def _patch_ensemble(s: str) -> str:
    def rep(a, b):
        nonlocal s
        assert s.count(a) == 1, f"ensemble source changed near: {a[:70]!r}"
        s = s.replace(a, b)
    rep("using namespace swg::sdev;\n", "using namespace swg::sdev;\nvoid swg_tr(cudaStream_t st, int id);\n")
    rep("    if (symba) {\n        const int64_t nmax = std::max(e->NPL, e->NTP);",
        "    if (symba) swg_tr(c->stream, 0);\n    if (symba) {\n        const int64_t nmax = std::max(e->NPL, e->NTP);")
    rep("            SWG_TRY(on_stream(c, e->side, [&] { return level0_launch(e, dt, sr, sv, st, stv); }));\n"
        "            SWG_TRY(vh2vb_pl(e, true));\n"
        "            SWG_TRY(lindrift_pl(e, dth, CB_PTBEG));\n"
        "            SWG_TRY(accel_int_pl(e, e->head));\n"
        "            SWG_TRY(on_stream(c, e->side, [&] { return level0_finish(e, dt); }));\n",
        "            SWG_TRY(on_stream(c, e->side, [&] { return level0_launch(e, dt, sr, sv, st, stv); }));\n"
        "            swg_tr(e->side, 1);\n"
        "            SWG_TRY(vh2vb_pl(e, true));\n"
        "            SWG_TRY(lindrift_pl(e, dth, CB_PTBEG));\n"
        "            swg_tr(c->stream, 2);\n"
        "            SWG_TRY(accel_int_pl(e, e->head));\n"
        "            swg_tr(c->stream, 3);\n"
        "            SWG_TRY(on_stream(c, e->side, [&] { return level0_finish(e, dt); }));\n"
        "            swg_tr(e->side, 4);\n")
    rep("    SWG_TRY(kick_vb_pl(e, dth, 1, have_acc));\n", "    SWG_TRY(kick_vb_pl(e, dth, 1, have_acc));\n"
        "    if (symba) swg_tr(c->stream, 5);\n")
    rep("        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), \"fork\"));\n"
        "        SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), \"fork\"));\n"
        "        SWG_TRY(recursion_launch(e, dt));\n"
        "        SWG_TRY(on_stream(c, e->side, [&] { return drift_bodies(e, dt); }));\n",
        "        swg_tr(c->stream, 6);\n"
        "        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_fork, c->stream), \"fork\"));\n"
        "        SWG_TRY(cuda_status(c, cudaStreamWaitEvent(e->side, e->ev_fork, 0), \"fork\"));\n"
        "        SWG_TRY(recursion_launch(e, dt));\n"
        "        swg_tr(c->stream, 7);\n"
        "        SWG_TRY(on_stream(c, e->side, [&] { return drift_bodies(e, dt); }));\n"
        "        swg_tr(e->side, 8);\n")
    rep("        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_join, e->side), \"join\"));\n"
        "        SWG_TRY(recursion_finish(e));\n",
        "        swg_tr(e->side, 9);\n"
        "        SWG_TRY(cuda_status(c, cudaEventRecord(e->ev_join, e->side), \"join\"));\n"
        "        SWG_TRY(recursion_finish(e));\n"
        "        swg_tr(c->stream, 10);\n")
    rep("            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), \"join\"));\n"
        "            SWG_TRY(kick_mixed_sym_reduce(",
        "            swg_tr(c->stream, 11);\n"
        "            SWG_TRY(cuda_status(c, cudaStreamWaitEvent(c->stream, e->ev_join, 0), \"join\"));\n"
        "            SWG_TRY(kick_mixed_sym_reduce(")
    rep("                                          e->sym_ppart, e->ah, 1, e->lany, 1, e->sym_tile, e->sym_group));\n",
        "                                          e->sym_ppart, e->ah, 1, e->lany, 1, e->sym_tile, e->sym_group));\n"
        "            swg_tr(c->stream, 12);\n")
    rep("        SWG_TRY(close_pl(e, dth, true));\n    } else {",
        "        SWG_TRY(close_pl(e, dth, true));\n        swg_tr(c->stream, 13);\n    } else {")
    rep("    k_ens_finish<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, symba ? e->lany : nullptr, e->lfirst,\n"
        "                                                                 e->enc_steps);\n"
        "    return L(c, \"ens_finish\");",
        "    k_ens_finish<<<grid_for(e->nsys, 128), 128, 0, c->stream>>>(e->nsys, symba ? e->lany : nullptr, e->lfirst,\n"
        "                                                                 e->enc_steps);\n"
        "    if (symba) swg_tr(c->stream, 14);\n"
        "    return L(c, \"ens_finish\");")
    return s + TRACE_DEF


def _patch_system(s: str) -> str:
    def rep(a, b):
        nonlocal s
        assert s.count(a) == 1, f"system source changed near: {a[:70]!r}"
        s = s.replace(a, b)
    rep("using namespace swg::sdev;\n", "using namespace swg::sdev;\nvoid swg_tr(cudaStream_t st, int id);\n")
    rep("    SWG_TRY(kick_vb_pl(s, dth, 1, !fork, opened));\n    SWG_TRY(drift_pl(s, dt));\n",
        "    SWG_TRY(kick_vb_pl(s, dth, 1, !fork, opened));\n    swg_tr(c->stream, 22);\n    SWG_TRY(drift_pl(s, dt));\n"
        "    swg_tr(c->stream, 23);\n")
    rep("            return drift_tp(s, dt);\n        }));\n",
        "            SWG_TRY(drift_tp(s, dt));\n            swg_tr(c->stream, 24);\n            return SWG_OK;\n        }));\n")
    rep("    SWG_TRY(symba_recursion(s, dt));\n    s->irec = -1;\n",
        "    SWG_TRY(symba_recursion(s, dt));\n    swg_tr(c->stream, 25);\n    s->irec = -1;\n")
    rep("        SWG_TRY(on_stream(c, s->side, [&] { return kick_vb_tp(s, dth, 0); }));\n",
        "        SWG_TRY(on_stream(c, s->side, [&] { SWG_TRY(kick_vb_tp(s, dth, 0)); swg_tr(c->stream, 27); "
        "return SWG_OK; }));\n")
    rep("    SWG_TRY(kick_vb_pl(s, dth, 0, !fork));\n    SWG_TRY(lindrift_pl(s, dth, 0));\n",
        "    SWG_TRY(kick_vb_pl(s, dth, 0, !fork));\n    swg_tr(c->stream, 26);\n    SWG_TRY(lindrift_pl(s, dth, 0));\n")
    rep("    s->lfirst_tp = s->lfirstkick;\n    s->lfirst_pl = s->lfirstkick;\n    int lany = 0;\n",
        "    swg_tr(c->stream, 20);\n    s->lfirst_tp = s->lfirstkick;\n    s->lfirst_pl = s->lfirstkick;\n"
        "    int lany = 0;\n")
    rep("    SWG_TRY(join(c, s->side, c->stream, s->ev[5]));\n    if (lany) {",
        "    SWG_TRY(join(c, s->side, c->stream, s->ev[5]));\n    swg_tr(c->stream, 21);\n    if (lany) {")
    rep("    s->lfirstkick = s->lfirst_pl;\n    return SWG_OK;\n}",
        "    s->lfirstkick = s->lfirst_pl;\n    swg_tr(c->stream, 28);\n    return SWG_OK;\n}")
    return s


def build() -> Path:
    from swiftest_gb300 import build as B
    src = ROOT / "swiftest_gb300" / "csrc"
    dst = ROOT / "_build" / "csrc_step_timeline"  # two levels down: the sources include ../../include
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(src, dst)
    p = dst / "ensemble.cu"
    p.write_text(_patch_ensemble(p.read_text()))
    q = dst / "system.cu"
    q.write_text(_patch_system(q.read_text()))
    B.CSRC, B.LIB, B.BUILD = dst, dst.parent / "libstep_timeline.so", dst.parent / "obj_step_timeline"
    return B.build(force=True)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c4", choices=["c4", "c1"])
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--skip", type=int, default=5, help="steps left out of the averages")
    ap.add_argument("--show", type=int, default=2)
    ap.add_argument("--nsys", type=int, default=None)
    args = ap.parse_args(argv)
    lib_path = build()
    from swiftest_gb300 import _lib
    _lib.LIB_PATH = lib_path
    import bench
    from swiftest_gb300.api import Context

    class A:
        encounter = "triangular"
        nsys = args.nsys

    wl = bench.C4(A) if args.workload == "c4" else bench.C1(A)
    ctx = Context(0)
    lib = _lib.load()
    lib.swg_trace_enable.argtypes = [C.c_int]
    lib.swg_trace_read.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    s = wl.make(ctx, "MIXED")
    s.step(3)
    first = 0 if args.workload == "c4" else 20
    cap = 1 << 16
    ids, g, h = np.zeros(cap, np.int32), np.zeros(cap, np.float32), np.zeros(cap, np.float64)
    steps = []
    for k in range(args.steps):
        lib.swg_trace_enable(1)
        s.step(1)
        lib.swg_trace_enable(0)
        n = lib.swg_trace_read(cap, ids.ctypes.data, g.ctypes.data, h.ctypes.data)
        rec = [(int(ids[i]), float(g[i]) * 1e3, float(h[i])) for i in range(n)]
        assert rec and rec[0][0] == first, rec[:3]
        steps.append(rec)
    s.close()
    ctx.close()
    out = {"workload": args.workload, "steps": args.steps, "skip": args.skip, "marks": {}, "last_steps": []}
    acc = {}
    for rec in steps[args.skip:]:
        for i, gu, hu in rec:
            acc.setdefault(i, []).append((gu, hu))
    for i in sorted(acc):
        a = np.array(acc[i])
        out["marks"][i] = {"name": MARKS[i][0], "stream": MARKS[i][1], "gpu_us_mean": round(float(a[:, 0].mean()), 1),
                           "host_us_mean": round(float(a[:, 1].mean()), 1), "count": len(a)}
    for rec in steps[-args.show:]:
        out["last_steps"].append([(MARKS[i][0], MARKS[i][1], round(gu, 1), round(hu, 1)) for i, gu, hu in rec])
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
