"""ctypes binding and build recipe for the CPU FP64 oracle (swiftest_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() as the
checker, and bench.py's CPU-baseline leg.  Parity unpinned by the reference's
own tests (it ships no kernel-level golden vectors and cannot be compiled
here); pinned instead by the known-answer tests in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "swiftest_oracle.c"
LIB = HERE / "liboracle.so"

# -ffp-contract=off: no fused multiply-adds (the GPU side builds with -fmad=false);
# no -march=native so x86 and aarch64 builds round identically.
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-fopenmp"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                                 (HERE / "swiftest_oracle.h").stat().st_mtime):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *CFLAGS, str(SRC), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64
_D = C.c_double
_SIG = {
    "orc_kick_getacch_int_all_tri_pl": (None, [_I32, _I32, _P, _P, _P, _P]),
    "orc_kick_getacch_int_all_flat_pl": (None, [_I32, _I64, _P, _P, _P, _P, _P]),
    "orc_kick_getacch_int_all_tp": (None, [_I32, _I32, _P, _P, _P, _P, _P]),
    "orc_util_flatten_eucl_plpl": (_I64, [_I32, _I32, _P]),
    "orc_el2xv": (None, [_I32, _P, _P, _P, _P]),
    "orc_xv2el": (None, [_I32, _P, _P, _P, _P]),
    "orc_drift_all": (None, [_P, _P, _P, _I32, _I32, _D, _D, _P, _P]),
    "orc_drift_all_count": (_I64, [_P, _P, _P, _I32, _D, _P, _P]),
    "orc_encounter_check_one": (None, [_D, _D, _D, _D, _D, _D, _D, _D, _P, _P]),
    "orc_encounter_check_all_plpl": (C.c_int, [C.c_int, _I32, _P, _P, _P, _D, _I64, C.POINTER(_I64), _P, _P, _P]),
    "orc_encounter_check_all_plplm": (C.c_int, [C.c_int, _I32, _I32, _P, _P, _P, _P, _P, _P, _D, _I64,
                                                C.POINTER(_I64), _P, _P, _P]),
    "orc_encounter_check_all_pltp": (C.c_int, [C.c_int, _I32, _I32, _P, _P, _P, _P, _P, _D, _I64, C.POINTER(_I64),
                                               _P, _P, _P]),
    "orc_system_create": (_P, [C.c_int, _I32, _I32]),
    "orc_system_destroy": (None, [_P]),
    "orc_system_set_cb": (None, [_P, _D, _D]),
    "orc_system_set_pl": (None, [_P, _P, _P, _P, _P, _P]),
    "orc_system_set_tp": (None, [_P, _P, _P]),
    "orc_system_set_param": (None, [_P, _D, C.c_int, C.c_int, C.c_int, _D, C.c_int, _D]),
    "orc_system_initialize": (C.c_int, [_P]),
    "orc_system_step": (C.c_int, [_P, _I32]),
    "orc_system_get_pl": (None, [_P, _P, _P, _P]),
    "orc_system_get_tp": (None, [_P, _P, _P, _P]),
    "orc_system_energy": (None, [_P, _P]),
    "orc_system_stats": (None, [_P, _P]),
    "orc_system_collision_terms": (None, [_P, _P]),
    "orc_system_plpl_list": (_I64, [_P, _I64, _P, _P]),
    "orc_system_pltp_list": (_I64, [_P, _I64, _P, _P]),
}
_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        for k, (r, a) in _SIG.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def kick_tri_pl(r, Gmass, radius=None, acc=None, nplm=None):
    lib = load()
    r = _f(r, (-1, 3))
    n = r.shape[0]
    acc = np.zeros((n, 3)) if acc is None else _f(acc, (n, 3)).copy()
    lib.orc_kick_getacch_int_all_tri_pl(n, n if nplm is None else nplm, _p(r), _p(_f(Gmass)),
                                        _p(None if radius is None else _f(radius)), _p(acc))
    return acc


def flatten(npl, nplm=None):
    lib = load()
    nplm = npl if nplm is None else nplm
    n = lib.orc_util_flatten_eucl_plpl(npl, nplm, None)
    k = np.zeros((max(n, 1), 2), np.int32)
    lib.orc_util_flatten_eucl_plpl(npl, nplm, _p(k))
    return k[:n]


def kick_flat_pl(r, Gmass, radius=None, acc=None, k_plpl=None, nplm=None):
    lib = load()
    r = _f(r, (-1, 3))
    n = r.shape[0]
    if k_plpl is None:
        k_plpl = flatten(n, nplm)
    k_plpl = np.ascontiguousarray(k_plpl, dtype=np.int32)
    acc = np.zeros((n, 3)) if acc is None else _f(acc, (n, 3)).copy()
    lib.orc_kick_getacch_int_all_flat_pl(n, k_plpl.shape[0], _p(k_plpl), _p(r), _p(_f(Gmass)),
                                         _p(None if radius is None else _f(radius)), _p(acc))
    return acc


def kick_tp(rtp, rpl, GMpl, lmask=None, acc=None):
    lib = load()
    rtp, rpl = _f(rtp, (-1, 3)), _f(rpl, (-1, 3))
    ntp = rtp.shape[0]
    m = np.ones(ntp, np.int32) if lmask is None else np.ascontiguousarray(lmask, dtype=np.int32)
    acc = np.zeros((ntp, 3)) if acc is None else _f(acc, (ntp, 3)).copy()
    lib.orc_kick_getacch_int_all_tp(ntp, rpl.shape[0], _p(rtp), _p(rpl), _p(_f(GMpl)), _p(m), _p(acc))
    return acc


ELEMENTS = ("a", "e", "inc", "capom", "omega", "capm", "varpi", "lam", "f", "cape", "capf")


def el2xv(mu, a, e, inc, capom, omega, capm):
    """swiftest_orbel_el2xv of every body: (rh, vh), each (n, 3)."""
    lib = load()
    a = np.ascontiguousarray(a, np.float64)
    n = len(a)
    mu = np.full(n, float(mu)) if np.isscalar(mu) else np.ascontiguousarray(mu, np.float64)
    el = np.ascontiguousarray(np.stack([a, e, inc, capom, omega, capm]), np.float64)
    rh, vh = np.zeros((n, 3)), np.zeros((n, 3))
    lib.orc_el2xv(n, _p(mu), _p(el), _p(rh), _p(vh))
    return rh, vh


def xv2el(mu, rh, vh):
    """swiftest_orbel_xv2el of every body: dict of the eleven element arrays."""
    lib = load()
    rh = np.ascontiguousarray(rh, np.float64).reshape(-1, 3)
    vh = np.ascontiguousarray(vh, np.float64).reshape(-1, 3)
    n = len(rh)
    mu = np.full(n, float(mu)) if np.isscalar(mu) else np.ascontiguousarray(mu, np.float64)
    out = np.zeros((11, n))
    lib.orc_xv2el(n, _p(mu), _p(rh), _p(vh), _p(out))
    return {k: out[i].copy() for i, k in enumerate(ELEMENTS)}


def drift_all(mu, x, v, dt, lmask=None, lgr=False, inv_c2=0.0):
    lib = load()
    x, v = _f(x, (-1, 3)).copy(), _f(v, (-1, 3)).copy()
    n = x.shape[0]
    mu = np.full(n, float(mu)) if np.isscalar(mu) else _f(mu)
    m = np.ones(n, np.int32) if lmask is None else np.ascontiguousarray(lmask, dtype=np.int32)
    iflag = np.zeros(n, np.int32)
    lib.orc_drift_all(_p(mu), _p(x), _p(v), n, int(bool(lgr)), float(inv_c2), float(dt), _p(m), _p(iflag))
    return x, v, iflag


def drift_stumpff_count(mu, x, v, dt):
    """Number of Stumpff evaluations for one drift of every body (FP64 work proxy)."""
    lib = load()
    x, v = _f(x, (-1, 3)).copy(), _f(v, (-1, 3)).copy()
    n = x.shape[0]
    mu = np.full(n, float(mu)) if np.isscalar(mu) else _f(mu)
    m = np.ones(n, np.int32)
    iflag = np.zeros(n, np.int32)
    return int(lib.orc_drift_all_count(_p(mu), _p(x), _p(v), n, float(dt), _p(m), _p(iflag)))


def encounter_one(xr, vr, renc, dt):
    lib = load()
    le, lv = C.c_int32(), C.c_int32()
    lib.orc_encounter_check_one(*map(float, xr), *map(float, vr), float(renc), float(dt), C.byref(le), C.byref(lv))
    return bool(le.value), bool(lv.value)


def _enc(fn, args):
    lib = load()
    cap = 1024
    n = C.c_int64()
    while True:
        i1, i2, lv = (np.zeros(cap, np.int32) for _ in range(3))
        rc = getattr(lib, fn)(*args, cap, C.byref(n), _p(i1), _p(i2), _p(lv))
        if rc == -3:
            cap = int(n.value)
            continue
        k = int(n.value)
        return i1[:k].copy(), i2[:k].copy(), lv[:k].astype(bool)


def encounter_plpl(r, v, renc, dt, mode=0):
    r, v = _f(r, (-1, 3)), _f(v, (-1, 3))
    return _enc("orc_encounter_check_all_plpl", [mode, r.shape[0], _p(r), _p(v), _p(_f(renc)), float(dt)])


def encounter_plplm(rplm, vplm, rplt, vplt, rencm, renct, dt, mode=0):
    rplm, vplm, rplt, vplt = (_f(a, (-1, 3)) for a in (rplm, vplm, rplt, vplt))
    return _enc("orc_encounter_check_all_plplm", [mode, rplm.shape[0], rplt.shape[0], _p(rplm), _p(vplm), _p(rplt),
                                                  _p(vplt), _p(_f(rencm)), _p(_f(renct)), float(dt)])


def encounter_pltp(rpl, vpl, rtp, vtp, renc, dt, mode=0):
    rpl, vpl, rtp, vtp = (_f(a, (-1, 3)) for a in (rpl, vpl, rtp, vtp))
    return _enc("orc_encounter_check_all_pltp", [mode, rpl.shape[0], rtp.shape[0], _p(rpl), _p(vpl), _p(rtp),
                                                 _p(vtp), _p(_f(renc)), float(dt)])


class OracleSystem:
    """CPU restatement of the reference's nbody system + step loops."""

    INTEGRATORS = {"WHM": 0, "HELIO": 1, "SYMBA": 2}

    def __init__(self, integrator, cb, pl, tp=None, dt=0.01, loop_mode="TRIANGULAR", encounter_check_plpl="TRIANGULAR",
                 encounter_check_pltp="TRIANGULAR", rhscale=6.5, lclose=True, gmtiny=0.0):
        lib = load()
        self.lib = lib
        npl = len(pl["Gmass"])
        ntp = 0 if tp is None else len(tp["rh"])
        self.npl, self.ntp = npl, ntp
        self.h = lib.orc_system_create(self.INTEGRATORS[integrator.upper()], npl, ntp)
        lib.orc_system_set_cb(self.h, float(cb["Gmass"]), float(cb["radius"]))
        if npl:
            arrs = [_f(pl["rh"], (npl, 3)), _f(pl["vh"], (npl, 3)), _f(pl["Gmass"]), _f(pl["radius"]),
                    _f(pl["rhill"])]
            lib.orc_system_set_pl(self.h, *map(_p, arrs))
        if ntp:
            lib.orc_system_set_tp(self.h, _p(_f(tp["rh"], (ntp, 3))), _p(_f(tp["vh"], (ntp, 3))))
        enc = {"TRIANGULAR": 0, "SORTSWEEP": 1}
        lib.orc_system_set_param(self.h, float(dt), {"TRIANGULAR": 0, "FLAT": 1}[loop_mode.upper()],
                                 enc[encounter_check_plpl.upper()], enc[encounter_check_pltp.upper()], float(rhscale),
                                 int(bool(lclose)), float(gmtiny))
        rc = lib.orc_system_initialize(self.h)
        if rc:
            raise RuntimeError(f"oracle initialize failed: {rc}")

    def step(self, n=1):
        rc = self.lib.orc_system_step(self.h, int(n))
        if rc:
            raise RuntimeError(f"oracle step failed: {rc}")

    def get_pl(self):
        rh, vh, st = np.zeros((self.npl, 3)), np.zeros((self.npl, 3)), np.zeros(self.npl, np.int32)
        self.lib.orc_system_get_pl(self.h, _p(rh), _p(vh), _p(st))
        return rh, vh, st

    def get_tp(self):
        rh, vh, st = np.zeros((self.ntp, 3)), np.zeros((self.ntp, 3)), np.zeros(self.ntp, np.int32)
        self.lib.orc_system_get_tp(self.h, _p(rh), _p(vh), _p(st))
        return rh, vh, st

    def energy(self):
        out = np.zeros(9)
        self.lib.orc_system_energy(self.h, _p(out))
        ct = np.zeros(4)
        self.lib.orc_system_collision_terms(self.h, _p(ct))
        return {"te": out[0], "ke": out[1], "pe": out[2], "be": out[3], "L": out[4:7].copy(), "GMtot": out[7],
                "te_helio": out[8], "E_collisions": ct[0], "L_escape": ct[1:4].copy()}

    def stats(self):
        out = np.zeros(6, np.int64)
        self.lib.orc_system_stats(self.h, _p(out))
        return {"steps_with_encounters": int(out[0]), "max_recursion": int(out[1]), "plpl_encounters": int(out[2]),
                "pltp_encounters": int(out[3]), "collisions": int(out[4]),
                "recursion_substeps": int(out[5])}

    def plpl_list(self):
        n = self.lib.orc_system_plpl_list(self.h, 0, None, None)
        i1, i2 = np.zeros(max(n, 1), np.int32), np.zeros(max(n, 1), np.int32)
        self.lib.orc_system_plpl_list(self.h, n, _p(i1), _p(i2))
        return i1[:n], i2[:n]

    def pltp_list(self):
        n = self.lib.orc_system_pltp_list(self.h, 0, None, None)
        i1, i2 = np.zeros(max(n, 1), np.int32), np.zeros(max(n, 1), np.int32)
        self.lib.orc_system_pltp_list(self.h, n, _p(i1), _p(i2))
        return i1[:n], i2[:n]

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_system_destroy(self.h)
                self.h = None
        except Exception:
            pass
