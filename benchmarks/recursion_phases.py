"""Cycles per SyMBA recursion sub-step, per phase, on the C1 system (mixed and FP64 steps).

    python benchmarks/recursion_phases.py [--steps 40]

Builds a copy of the library (under _build/) whose recursion kernel reads the
SM clock (clock64) at the boundaries of its phases (list check, the two kicks, the drift, the
collision check, the level reset, loop control) and adds the intervals of thread 0 to a device
array, then steps the seeded C1 disk (2000 pl + 10000 tp) and prints the cycles per sub-step of
each phase.  The timers only read the clock between the phases' barriers; the phases' work is
unchanged.  Measurement tool: the product library is not touched.
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

NAMES = ["setup", "list_check", "kick1", "drift", "kick2", "coll_check", "set_levels", "loop_pre", "pre_kick2",
         "tail", "substeps", "stage_load"]


def _patch(s: str) -> str:
    def rep(a, b):
        nonlocal s
        assert s.count(a) == 1, f"recursion source changed near: {a[:60]!r}"
        s = s.replace(a, b)
    rep("template <bool STAGED>\nstatic __device__ void blk_symba_recursion_t(const RecArgs &a, void *stage) {",
        "__device__ unsigned long long g_ph[16];\n"
        "#define PH(k, t0) if (threadIdx.x == 0) { unsigned long long _n = clock64(); "
        "atomicAdd(&g_ph[k], _n - t0); t0 = _n; }\n"
        "template <bool STAGED>\nstatic __device__ void blk_symba_recursion_t(const RecArgs &a, void *stage) {\n"
        "    unsigned long long t0 = clock64();")
    rep("    blk_build_adjacency(a, nbpl, nbtp);\n    RecStage S{};",
        "    blk_build_adjacency(a, nbpl, nbtp);\n    PH(0, t0)\n    RecStage S{};")
    rep("        stg_load(a, S, nbpl, nbtp);\n    }", "        stg_load(a, S, nbpl, nbtp);\n    }\n    PH(11, t0)")
    for call, k in (("stg_list_check(a, S, irecp, dtl, &s_any, s_rs);", 1),
                    ("stg_kick_lists(a, S, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);\n                stg_drift", 2),
                    ("stg_drift(a, S, nbpl, nbtp, ireci, dtl, inv_gm);", 3),
                    ("blk_list_check(a, irecp, dtl, &s_any, s_rs);", 1),
                    ("blk_kick_lists(a, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);\n                blk_drift", 2),
                    ("blk_drift(a, nbpl, nbtp, ireci, dtl, inv_gm);", 3)):
        if call.endswith("stg_drift") or call.endswith("blk_drift"):
            head, tail = call.split("\n")
            rep(call, f"{head}\n                PH({k}, t0)\n{tail}")
        else:
            rep(call, f"{call}\n                PH({k}, t0)")
    rep("            const int any = s_any;",
        "            if (threadIdx.x == 0) atomicAdd(&g_ph[10], 1ull);\n            const int any = s_any;")
    rep("        // after the deeper levels (or none) for loop j of level ireci\n",
        "        // after the deeper levels (or none) for loop j of level ireci\n        PH(8, t0)\n")
    rep("            blk_kick_lists(a, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);\n        if (a.lclose) {",
        "            blk_kick_lists(a, nbpl, nbtp, dth, irecp, ireci != 0, s_pw);\n        PH(4, t0)\n"
        "        if (a.lclose) {")
    rep("                blk_collision_check(a, ireci, dtl, &s_any);",
        "                blk_collision_check(a, ireci, dtl, &s_any);\n            PH(5, t0)")
    rep("            blk_set_recur_levels(a, nbpl, nbtp, ireci);\n        if (threadIdx.x == 0) {",
        "            blk_set_recur_levels(a, nbpl, nbtp, ireci);\n        PH(6, t0)\n        if (threadIdx.x == 0) {")
    rep("    if constexpr (STAGED) stg_store(a, S, nbpl, nbtp);",
        "    PH(9, t0)\n    if constexpr (STAGED) stg_store(a, S, nbpl, nbtp);")
    # loop control: from the end of the previous phase to the list check
    rep("            if (threadIdx.x == 0) s_any = 0;\n            __syncthreads();\n            if constexpr (STAGED) {",
        "            if (threadIdx.x == 0) s_any = 0;\n            __syncthreads();\n            PH(7, t0)\n"
        "            if constexpr (STAGED) {")
    return s


def build() -> Path:
    from swiftest_gb300 import build as B
    src = ROOT / "swiftest_gb300" / "csrc"
    dst = ROOT / "_build" / "csrc_recursion_phases"  # two levels down: the sources include ../../include
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(src, dst)
    p = dst / "symba_dev.cuh"
    p.write_text(_patch(p.read_text()))
    q = dst / "system.cu"
    q.write_text(q.read_text() + """
extern "C" int swg_probe_recursion_phases(unsigned long long *out) {
    cudaDeviceSynchronize();
    cudaMemcpyFromSymbol(out, g_ph, sizeof(unsigned long long) * 16);
    unsigned long long z[16] = {0};
    cudaMemcpyToSymbol(g_ph, z, sizeof(z));
    return 0;
}
""")
    B.CSRC, B.LIB, B.BUILD = dst, dst.parent / "librecursion_phases.so", dst.parent / "obj_recursion_phases"
    return B.build(force=True)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=40)
    args = ap.parse_args(argv)
    lib_path = build()
    from swiftest_gb300 import _lib
    _lib.LIB_PATH = lib_path
    import bench
    from swiftest_gb300.api import Context

    class A:
        encounter = "triangular"

    wl = bench.C1(A)
    ctx = Context(0)
    lib = _lib.load()
    fn = lib.swg_probe_recursion_phases
    fn.argtypes = [C.c_void_p]
    buf = np.zeros(16, np.uint64)
    out = {}
    for prec in ("MIXED", "FP64"):
        s = wl.make(ctx, prec)
        fn(buf.ctypes.data)
        tot = np.zeros(16)
        for _ in range(args.steps):
            s.step(1)
            fn(buf.ctypes.data)
            tot += buf
        s.close()
        sub = max(tot[10], 1.0)
        per = {n: round(float(tot[i]) / sub) for i, n in enumerate(NAMES) if n != "substeps"}
        out[prec] = {"substeps": int(tot[10]), "cycles_per_substep": per,
                     "total": round(float(sum(tot[:10]) + tot[11]) / sub)}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
