"""Python host layer over the C ABI: numpy in, numpy out.

Names and argument meanings follow the reference's Fortran procedures
(src/swiftest/swiftest_module.f90:505-539, 924-1010; src/encounter/encounter_module.f90).
Arrays use the reference layout: positions/velocities of shape (n, 3) in C
order, which is the same memory as Fortran's (3, n); encounter indices are
1-based; masks are int32 0/1.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib as L


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One CUDA stream plus a grow-only device arena (``swg_ctx``)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        rc = self.lib.swg_create(C.byref(h), device)
        if rc != L.SWG_OK:
            raise L.SwiftestGB300Error("swg_create", rc, "no usable CUDA device")
        self.h = h
        self._systems = weakref.WeakSet()

    def close(self):
        # the C context destroys the systems and ensembles still attached to it; mark them closed
        for s in list(getattr(self, "_systems", ())):
            s.h = None
        if getattr(self, "h", None):
            self.lib.swg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, fn: str, rc: int):
        if rc != L.SWG_OK:
            msg = self.lib.swg_last_error(self.h)
            raise L.SwiftestGB300Error(fn, rc, msg.decode() if msg else "")

    @property
    def launches(self) -> int:
        return int(self.lib.swg_launch_count(self.h))

    def synchronize(self):
        self.check("swg_synchronize", self.lib.swg_synchronize(self.h))

    # ---- measurement helpers ---------------------------------------------
    def flush_l2(self, nbytes: int = 512 << 20):
        self.check("swg_flush_l2", self.lib.swg_flush_l2(self.h, int(nbytes)))

    def event_record(self, slot: int):
        self.check("swg_event_record", self.lib.swg_event_record(self.h, int(slot)))

    def event_elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double()
        self.check("swg_event_elapsed", self.lib.swg_event_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return float(ms.value)

    def probe_peak_tflops(self, kind: str = "fp32") -> float:
        t = C.c_double()
        k = {"fp32": 0, "fp64": 1, "fp32x2": 2}[kind]
        self.check("swg_probe_peak", self.lib.swg_probe_peak(self.h, k, C.byref(t)))
        return float(t.value)

    # ---- kick -------------------------------------------------------------
    def kick_getacch_int_all_tri_pl(self, r, Gmass, radius=None, acc=None, nplm=None, precision=L.SWG_FP64):
        r = _f64(r, (-1, 3))
        npl = r.shape[0]
        acc = np.zeros((npl, 3)) if acc is None else _f64(acc, (npl, 3)).copy()
        nplm = npl if nplm is None else int(nplm)
        g = _f64(Gmass)
        rad = None if radius is None else _f64(radius)
        rc = self.lib.swg_kick_getacch_int_all_tri_pl(self.h, npl, nplm, _ptr(r), _ptr(g), _ptr(rad), _ptr(acc),
                                                      precision, L.SWG_MEM_HOST)
        self.check("swg_kick_getacch_int_all_tri_pl", rc)
        return acc

    def kick_getacch_int_all_flat_pl(self, r, Gmass, radius=None, acc=None, k_plpl=None, nplm=None,
                                     precision=L.SWG_FP64):
        r = _f64(r, (-1, 3))
        npl = r.shape[0]
        nplm = npl if nplm is None else int(nplm)
        acc = np.zeros((npl, 3)) if acc is None else _f64(acc, (npl, 3)).copy()
        g = _f64(Gmass)
        rad = None if radius is None else _f64(radius)
        if k_plpl is None:
            nplpl = nplm * npl - nplm * (nplm + 1) // 2
            kp = None
        else:
            kp = _i32(k_plpl).reshape(-1, 2)
            nplpl = kp.shape[0]
        rc = self.lib.swg_kick_getacch_int_all_flat_pl(self.h, npl, nplm, nplpl, _ptr(kp), _ptr(r), _ptr(g),
                                                       _ptr(rad), _ptr(acc), precision, L.SWG_MEM_HOST)
        self.check("swg_kick_getacch_int_all_flat_pl", rc)
        return acc

    def kick_getacch_int_all_tp(self, rtp, rpl, GMpl, lmask=None, acc=None, precision=L.SWG_FP64):
        rtp = _f64(rtp, (-1, 3))
        rpl = _f64(rpl, (-1, 3))
        ntp, npl = rtp.shape[0], rpl.shape[0]
        acc = np.zeros((ntp, 3)) if acc is None else _f64(acc, (ntp, 3)).copy()
        m = np.ones(ntp, np.int32) if lmask is None else _i32(lmask)
        g = _f64(GMpl)
        rc = self.lib.swg_kick_getacch_int_all_tp(self.h, ntp, npl, _ptr(rtp), _ptr(rpl), _ptr(g), _ptr(m),
                                                  _ptr(acc), precision, L.SWG_MEM_HOST)
        self.check("swg_kick_getacch_int_all_tp", rc)
        return acc

    # ---- drift ------------------------------------------------------------
    def drift_all(self, mu, x, v, dt, lmask=None, lgr=False, inv_c2=0.0):
        x = _f64(x, (-1, 3)).copy()
        v = _f64(v, (-1, 3)).copy()
        n = x.shape[0]
        mu = np.full(n, float(mu)) if np.isscalar(mu) else _f64(mu)
        m = np.ones(n, np.int32) if lmask is None else _i32(lmask)
        iflag = np.zeros(n, np.int32)
        rc = self.lib.swg_drift_all(self.h, _ptr(mu), _ptr(x), _ptr(v), n, int(bool(lgr)), float(inv_c2), float(dt),
                                    _ptr(m), _ptr(iflag), L.SWG_MEM_HOST)
        self.check("swg_drift_all", rc)
        return x, v, iflag

    def util_sort_index(self, arr):
        """util_sort(arr, ind): the 1-based permutation that sorts arr ascending (ties by index)."""
        a = _f64(arr)
        ind = np.zeros(a.shape[0], np.int32)
        self.check("swg_util_sort_index", self.lib.swg_util_sort_index(self.h, a.shape[0], _ptr(a), _ptr(ind),
                                                                       L.SWG_MEM_HOST))
        return ind

    # ---- orbital elements ----------------------------------------------------
    ELEMENTS = ("a", "e", "inc", "capom", "omega", "capm", "varpi", "lam", "f", "cape", "capf")

    def el2xv(self, mu, a, e, inc, capom, omega, capm):
        """Heliocentric positions and velocities (n, 3) from orbital elements (radians)."""
        a = _f64(a)
        n = a.shape[0]
        mu = np.full(n, float(mu)) if np.isscalar(mu) else _f64(mu)
        els = [_f64(x) for x in (e, inc, capom, omega, capm)]
        rh, vh = np.zeros((n, 3)), np.zeros((n, 3))
        rc = self.lib.swg_orbel_el2xv(self.h, n, _ptr(mu), _ptr(a), *[_ptr(x) for x in els], _ptr(rh), _ptr(vh),
                                      L.SWG_MEM_HOST)
        self.check("swg_orbel_el2xv", rc)
        return rh, vh

    def xv2el(self, mu, rh, vh):
        """Orbital elements of (n, 3) positions and velocities: dict of the eleven arrays."""
        rh = _f64(rh, (-1, 3))
        vh = _f64(vh, (-1, 3))
        n = rh.shape[0]
        mu = np.full(n, float(mu)) if np.isscalar(mu) else _f64(mu)
        out = {k: np.zeros(n) for k in self.ELEMENTS}
        rc = self.lib.swg_orbel_xv2el(self.h, n, _ptr(mu), _ptr(rh), _ptr(vh), *[_ptr(out[k]) for k in self.ELEMENTS],
                                      L.SWG_MEM_HOST)
        self.check("swg_orbel_xv2el", rc)
        return out

    # ---- encounters -------------------------------------------------------
    def _enc(self, fn, args, cap):
        n = C.c_int64(0)
        while True:
            i1 = np.zeros(max(cap, 1), np.int32)
            i2 = np.zeros(max(cap, 1), np.int32)
            lv = np.zeros(max(cap, 1), np.int32)
            rc = getattr(self.lib, fn)(self.h, *args, cap, C.byref(n), _ptr(i1), _ptr(i2), _ptr(lv), L.SWG_MEM_HOST)
            if rc == L.SWG_ERR_CAPACITY:
                cap = int(n.value)
                continue
            self.check(fn, rc)
            k = int(n.value)
            return i1[:k].copy(), i2[:k].copy(), lv[:k].astype(bool)

    def encounter_check_all_plpl(self, r, v, renc, dt, mode=L.SWG_ENC_TRIANGULAR, cap=1024):
        r = _f64(r, (-1, 3))
        v = _f64(v, (-1, 3))
        renc = _f64(renc)
        return self._enc("swg_encounter_check_all_plpl",
                         [mode, r.shape[0], _ptr(r), _ptr(v), _ptr(renc), float(dt)], cap)

    def encounter_check_all_plplm(self, rplm, vplm, rplt, vplt, rencm, renct, dt, mode=L.SWG_ENC_TRIANGULAR,
                                  cap=1024):
        rplm, vplm = _f64(rplm, (-1, 3)), _f64(vplm, (-1, 3))
        rplt, vplt = _f64(rplt, (-1, 3)), _f64(vplt, (-1, 3))
        rencm, renct = _f64(rencm), _f64(renct)
        return self._enc("swg_encounter_check_all_plplm",
                         [mode, rplm.shape[0], rplt.shape[0], _ptr(rplm), _ptr(vplm), _ptr(rplt), _ptr(vplt),
                          _ptr(rencm), _ptr(renct), float(dt)], cap)

    def encounter_check_all_pltp(self, rpl, vpl, rtp, vtp, renc, dt, mode=L.SWG_ENC_TRIANGULAR, cap=1024):
        rpl, vpl = _f64(rpl, (-1, 3)), _f64(vpl, (-1, 3))
        rtp, vtp = _f64(rtp, (-1, 3)), _f64(vtp, (-1, 3))
        renc = _f64(renc)
        return self._enc("swg_encounter_check_all_pltp",
                         [mode, rpl.shape[0], rtp.shape[0], _ptr(rpl), _ptr(vpl), _ptr(rtp), _ptr(vtp), _ptr(renc),
                          float(dt)], cap)


INTEGRATORS = {"WHM": L.SWG_WHM, "HELIO": L.SWG_HELIO, "SYMBA": L.SWG_SYMBA}


class NBodySystem:
    """Device-resident n-body system stepped by the WHM / HELIO / SyMBA loops.

    Mirrors ``swiftest_nbody_system`` + ``step`` (src/swiftest/swiftest_driver.f90:130-180).
    Massive bodies must already be ordered as the reference's initialise does
    (HELIO/SyMBA: Gmass descending; WHM: heliocentric distance ascending), which
    ``initial_conditions.sort_for_integrator`` provides.
    """

    def __init__(self, ctx: Context, integrator: str, cb, pl, tp=None, dt=0.01, loop_mode="TRIANGULAR",
                 encounter_check_plpl="TRIANGULAR", encounter_check_pltp="TRIANGULAR", rhscale=6.5, lclose=True,
                 gmtiny=0.0, precision="FP64"):
        self.ctx = ctx
        lib = ctx.lib
        self.integrator = integrator.upper()
        npl = len(pl["Gmass"])
        ntp = 0 if tp is None else len(tp["rh"])
        h = C.c_void_p()
        ctx.check("swg_system_create", lib.swg_system_create(ctx.h, INTEGRATORS[self.integrator], npl, ntp,
                                                             C.byref(h)))
        self.h = h
        ctx._systems.add(self)
        self.npl, self.ntp = npl, ntp
        ctx.check("swg_system_set_cb", lib.swg_system_set_cb(h, float(cb["Gmass"]), float(cb["radius"])))
        self._keep = []
        if npl:
            arrs = [_f64(pl["rh"], (npl, 3)), _f64(pl["vh"], (npl, 3)), _f64(pl["Gmass"]), _f64(pl["radius"]),
                    _f64(pl["rhill"])]
            ctx.check("swg_system_set_pl", lib.swg_system_set_pl(h, *[_ptr(a) for a in arrs]))
        if ntp:
            arrs = [_f64(tp["rh"], (ntp, 3)), _f64(tp["vh"], (ntp, 3))]
            ctx.check("swg_system_set_tp", lib.swg_system_set_tp(h, *[_ptr(a) for a in arrs]))
        enc = {"TRIANGULAR": L.SWG_ENC_TRIANGULAR, "SORTSWEEP": L.SWG_ENC_SORTSWEEP}
        loop = {"TRIANGULAR": 0, "FLAT": 1}[loop_mode.upper()]
        prec = {"FP64": L.SWG_FP64, "MIXED": L.SWG_MIXED}[precision.upper()]
        ctx.check("swg_system_set_param", lib.swg_system_set_param(
            h, float(dt), loop, enc[encounter_check_plpl.upper()], enc[encounter_check_pltp.upper()], float(rhscale),
            int(bool(lclose)), float(gmtiny), prec))
        ctx.check("swg_system_initialize", lib.swg_system_initialize(h))

    def step(self, nsteps: int = 1):
        self.ctx.check("swg_system_step", self.ctx.lib.swg_system_step(self.h, int(nsteps)))

    def set_state(self, rh=None, vh=None, trh=None, tvh=None):
        """Upload positions / heliocentric velocities (host arrays) without resetting step
        flags; a changed state reaches the next step after reset_first_step."""
        self.ctx.check("swg_system_set_state", self.ctx.lib.swg_system_set_state(
            self.h, _ptr(rh), _ptr(vh), _ptr(trh), _ptr(tvh)))

    def get_state_async(self, rh=None, vh=None, trh=None, tvh=None):
        self.ctx.check("swg_system_get_state_async", self.ctx.lib.swg_system_get_state_async(
            self.h, _ptr(rh), _ptr(vh), _ptr(trh), _ptr(tvh)))

    def reset_first_step(self):
        """Set the first-step flags (the reference's lfirst): the next step takes the
        uploaded vh and evaluates its opening accelerations afresh (see set_state)."""
        self.ctx.check("swg_system_reset_first_step", self.ctx.lib.swg_system_reset_first_step(self.h))

    PROFILE_CLASSES = ("kick_pl", "kick_tp", "drift", "encounter_level0", "symba_recursion")

    def profile(self, enable: bool = True):
        self.ctx.check("swg_system_profile", self.ctx.lib.swg_system_profile(self.h, int(bool(enable))))

    def profile_read(self):
        out = np.zeros(10)
        self.ctx.check("swg_system_profile_read", self.ctx.lib.swg_system_profile_read(self.h, _ptr(out)))
        return {k: {"launches": int(out[2 * i]), "ms": float(out[2 * i + 1])}
                for i, k in enumerate(self.PROFILE_CLASSES)}

    def get_pl(self):
        rh = np.zeros((self.npl, 3))
        vh = np.zeros((self.npl, 3))
        st = np.zeros(self.npl, np.int32)
        self.ctx.check("swg_system_get_pl", self.ctx.lib.swg_system_get_pl(self.h, _ptr(rh), _ptr(vh), _ptr(st)))
        return rh, vh, st

    def get_pl_masses(self):
        """Current Gmass, radius and rhill of the massive bodies (merges change them)."""
        g, r, h = np.zeros(self.npl), np.zeros(self.npl), np.zeros(self.npl)
        self.ctx.check("swg_system_get_pl_masses",
                       self.ctx.lib.swg_system_get_pl_masses(self.h, _ptr(g), _ptr(r), _ptr(h)))
        return g, r, h

    def get_tp(self):
        rh = np.zeros((self.ntp, 3))
        vh = np.zeros((self.ntp, 3))
        st = np.zeros(self.ntp, np.int32)
        self.ctx.check("swg_system_get_tp", self.ctx.lib.swg_system_get_tp(self.h, _ptr(rh), _ptr(vh), _ptr(st)))
        return rh, vh, st

    def energy(self):
        out = np.zeros(9)
        self.ctx.check("swg_system_energy", self.ctx.lib.swg_system_energy(self.h, _ptr(out)))
        ct = np.zeros(4)
        self.ctx.check("swg_system_collision_terms", self.ctx.lib.swg_system_collision_terms(self.h, _ptr(ct)))
        return {"te": out[0], "ke": out[1], "pe": out[2], "be": out[3], "L": out[4:7].copy(), "GMtot": out[7],
                "te_helio": out[8], "E_collisions": ct[0], "L_escape": ct[1:4].copy()}

    def stats(self):
        out = np.zeros(6, np.int64)
        self.ctx.check("swg_system_stats", self.ctx.lib.swg_system_stats(self.h, _ptr(out)))
        return {"steps_with_encounters": int(out[0]), "max_recursion": int(out[1]), "plpl_encounters": int(out[2]),
                "pltp_encounters": int(out[3]), "collisions": int(out[4]),
                "recursion_substeps": int(out[5])}

    def _list(self, fn):
        n = C.c_int64(0)
        cap = 1024
        while True:
            i1 = np.zeros(cap, np.int32)
            i2 = np.zeros(cap, np.int32)
            rc = getattr(self.ctx.lib, fn)(self.h, cap, C.byref(n), _ptr(i1), _ptr(i2))
            if rc == L.SWG_ERR_CAPACITY:
                cap = int(n.value)
                continue
            self.ctx.check(fn, rc)
            return i1[:n.value].copy(), i2[:n.value].copy()

    def plpl_list(self):
        return self._list("swg_system_plpl_list")

    def pltp_list(self):
        return self._list("swg_system_pltp_list")

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.ctx.lib.swg_system_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Many independent systems stepped together (``swg_ensemble``), CSR-packed.

    ``ens`` is the dict of ``initial_conditions.make_ensemble``: per-system ``npl``,
    ``ntp``, ``GMcb``, ``Rcb`` and the concatenated, per-system sorted body arrays.
    Each system takes exactly the steps of ``NBodySystem`` with the same integrator
    (bit-identical with precision="FP64").
    """

    PROFILE_CLASSES = NBodySystem.PROFILE_CLASSES

    def __init__(self, ctx: Context, ens: dict, dt=None, rhscale=None, lclose=True, precision="FP64",
                 encounter_check_plpl="TRIANGULAR", encounter_check_pltp="TRIANGULAR", gmtiny=0.0):
        self.ctx = ctx
        lib = ctx.lib
        self.integrator = ens["integrator"].upper()
        self.npl = _i32(ens["npl"])
        self.ntp = _i32(ens["ntp"])
        self.nsys = len(self.npl)
        self.NPL, self.NTP = int(self.npl.sum()), int(self.ntp.sum())
        self.poff = np.concatenate([[0], np.cumsum(self.npl)]).astype(np.int64)
        self.toff = np.concatenate([[0], np.cumsum(self.ntp)]).astype(np.int64)
        h = C.c_void_p()
        ctx.check("swg_ensemble_create", lib.swg_ensemble_create(ctx.h, INTEGRATORS[self.integrator], self.nsys,
                                                                 _ptr(self.npl), _ptr(self.ntp), C.byref(h)))
        self.h = h
        ctx._systems.add(self)
        ctx.check("swg_ensemble_set_cb", lib.swg_ensemble_set_cb(h, _ptr(_f64(ens["GMcb"])), _ptr(_f64(ens["Rcb"]))))
        pl, tp = ens["pl"], ens["tp"]
        if self.NPL:
            arrs = [_f64(pl["rh"], (self.NPL, 3)), _f64(pl["vh"], (self.NPL, 3)), _f64(pl["Gmass"]),
                    _f64(pl["radius"]), _f64(pl["rhill"])]
            ctx.check("swg_ensemble_set_pl", lib.swg_ensemble_set_pl(h, *[_ptr(a) for a in arrs]))
        if self.NTP:
            arrs = [_f64(tp["rh"], (self.NTP, 3)), _f64(tp["vh"], (self.NTP, 3))]
            ctx.check("swg_ensemble_set_tp", lib.swg_ensemble_set_tp(h, *[_ptr(a) for a in arrs]))
        prec = {"FP64": L.SWG_FP64, "MIXED": L.SWG_MIXED}[precision.upper()]
        ctx.check("swg_ensemble_set_param", lib.swg_ensemble_set_param(
            h, float(ens["dt"] if dt is None else dt), float(ens["rhscale"] if rhscale is None else rhscale),
            int(bool(lclose)), prec))
        modes = {"TRIANGULAR": L.SWG_ENC_TRIANGULAR, "SORTSWEEP": L.SWG_ENC_SORTSWEEP}
        m = (modes[encounter_check_plpl.upper()], modes[encounter_check_pltp.upper()])
        if m != (L.SWG_ENC_TRIANGULAR, L.SWG_ENC_TRIANGULAR):
            ctx.check("swg_ensemble_set_encounter_modes", lib.swg_ensemble_set_encounter_modes(h, *m))
        if gmtiny:
            ctx.check("swg_ensemble_set_gmtiny", lib.swg_ensemble_set_gmtiny(h, float(gmtiny)))
        ctx.check("swg_ensemble_initialize", lib.swg_ensemble_initialize(h))

    def step(self, nsteps: int = 1):
        self.ctx.check("swg_ensemble_step", self.ctx.lib.swg_ensemble_step(self.h, int(nsteps)))

    def set_state(self, rh=None, vh=None, trh=None, tvh=None):
        self.ctx.check("swg_ensemble_set_state", self.ctx.lib.swg_ensemble_set_state(
            self.h, _ptr(rh), _ptr(vh), _ptr(trh), _ptr(tvh)))

    def get_state_async(self, rh=None, vh=None, trh=None, tvh=None):
        self.ctx.check("swg_ensemble_get_state_async", self.ctx.lib.swg_ensemble_get_state_async(
            self.h, _ptr(rh), _ptr(vh), _ptr(trh), _ptr(tvh)))

    def reset_first_step(self):
        """Set every system's first-step flags (the reference's lfirst), as
        NBodySystem.reset_first_step does for one system."""
        self.ctx.check("swg_ensemble_reset_first_step", self.ctx.lib.swg_ensemble_reset_first_step(self.h))

    def get_pl(self):
        rh = np.zeros((self.NPL, 3))
        vh = np.zeros((self.NPL, 3))
        st = np.zeros(self.NPL, np.int32)
        self.ctx.check("swg_ensemble_get_pl", self.ctx.lib.swg_ensemble_get_pl(self.h, _ptr(rh), _ptr(vh), _ptr(st)))
        return rh, vh, st

    def get_pl_masses(self):
        """Current Gmass, radius and rhill of every system's massive bodies (CSR order)."""
        g, r, h = np.zeros(self.NPL), np.zeros(self.NPL), np.zeros(self.NPL)
        self.ctx.check("swg_ensemble_get_pl_masses",
                       self.ctx.lib.swg_ensemble_get_pl_masses(self.h, _ptr(g), _ptr(r), _ptr(h)))
        return g, r, h

    def get_tp(self):
        rh = np.zeros((self.NTP, 3))
        vh = np.zeros((self.NTP, 3))
        st = np.zeros(self.NTP, np.int32)
        self.ctx.check("swg_ensemble_get_tp", self.ctx.lib.swg_ensemble_get_tp(self.h, _ptr(rh), _ptr(vh), _ptr(st)))
        return rh, vh, st

    def energy(self):
        """Per-system energy / momentum: dict of arrays (length nsys)."""
        out = np.zeros((self.nsys, 9))
        self.ctx.check("swg_ensemble_energy", self.ctx.lib.swg_ensemble_energy(self.h, _ptr(out)))
        ct = np.zeros((self.nsys, 4))
        self.ctx.check("swg_ensemble_collision_terms",
                       self.ctx.lib.swg_ensemble_collision_terms(self.h, _ptr(ct)))
        return {"te": out[:, 0].copy(), "ke": out[:, 1].copy(), "pe": out[:, 2].copy(), "be": out[:, 3].copy(),
                "L": out[:, 4:7].copy(), "GMtot": out[:, 7].copy(), "te_helio": out[:, 8].copy(),
                "E_collisions": ct[:, 0].copy(), "L_escape": ct[:, 1:4].copy()}

    def stats(self):
        out = np.zeros(6, np.int64)
        self.ctx.check("swg_ensemble_stats", self.ctx.lib.swg_ensemble_stats(self.h, _ptr(out)))
        return {"system_steps_with_encounters": int(out[0]), "max_recursion": int(out[1]),
                "plpl_encounters": int(out[2]), "pltp_encounters": int(out[3]), "collisions": int(out[4]),
                "recursion_substeps": int(out[5])}

    def plpl_list(self, sys: int):
        n = C.c_int64(0)
        cap = 256
        while True:
            i1 = np.zeros(cap, np.int32)
            i2 = np.zeros(cap, np.int32)
            rc = self.ctx.lib.swg_ensemble_plpl_list(self.h, int(sys), cap, C.byref(n), _ptr(i1), _ptr(i2))
            if rc == L.SWG_ERR_CAPACITY:
                cap = int(n.value)
                continue
            self.ctx.check("swg_ensemble_plpl_list", rc)
            return i1[:n.value].copy(), i2[:n.value].copy()

    def use_graphs(self, enable: bool = True):
        self.ctx.check("swg_ensemble_use_graphs", self.ctx.lib.swg_ensemble_use_graphs(self.h, int(bool(enable))))

    def set_kick_variant(self, variant: int = -1):
        """Force a broadcast tile shape (0 .. SWG_KICK_NVARIANT-1) on both mixed kicks, or
        use the default (-1): symmetric pl-pl kernel, autotuned pl-tp shape."""
        self.ctx.check("swg_ensemble_set_kick_variant", self.ctx.lib.swg_ensemble_set_kick_variant(self.h, int(variant)))

    def set_kick_strip(self, strip: int = 0):
        """Force the symmetric pl-pl kick's strip length (1, 2, 4, 8 or 16 tile pairs per
        item), or let the autotuner choose it (0)."""
        self.ctx.check("swg_ensemble_set_kick_strip", self.ctx.lib.swg_ensemble_set_kick_strip(self.h, int(strip)))

    def kick_strip(self) -> int:
        """Strip length of the symmetric pl-pl kick in use (-1 before the first mixed kick)."""
        v = C.c_int(-1)
        self.ctx.check("swg_ensemble_kick_variant", self.ctx.lib.swg_ensemble_kick_variant(self.h, 2, C.byref(v)))
        return int(v.value)

    def set_kick_warps(self, warps: int = 0):
        """Force the symmetric pl-pl kick's warps per block (1, 2 or 4; the same bits for
        each), or let the autotuner choose it (0)."""
        self.ctx.check("swg_ensemble_set_kick_warps", self.ctx.lib.swg_ensemble_set_kick_warps(self.h, int(warps)))

    def set_kick_tile(self, tile: int = 0):
        """Force the symmetric pl-pl kick's bodies per tile (128 or 64), or let the autotuner
        choose it (0)."""
        self.ctx.check("swg_ensemble_set_kick_tile", self.ctx.lib.swg_ensemble_set_kick_tile(self.h, int(tile)))

    def kick_tile(self) -> int:
        """Bodies per tile of the symmetric pl-pl kick in use (-1 before the first mixed kick)."""
        v = C.c_int(-1)
        self.ctx.check("swg_ensemble_kick_variant", self.ctx.lib.swg_ensemble_kick_variant(self.h, 4, C.byref(v)))
        return int(v.value)

    def set_kick_group(self, group: int = 0):
        """Force the symmetric pl-pl kick's tiles per row group (1, 2 or 4; groups take
        128-body tiles and a block of that many warps per item), or let the autotuner choose
        it (0)."""
        self.ctx.check("swg_ensemble_set_kick_group", self.ctx.lib.swg_ensemble_set_kick_group(self.h, int(group)))

    def kick_group(self) -> int:
        """Tiles per row group of the symmetric pl-pl kick in use (-1 before the first mixed kick)."""
        v = C.c_int(-1)
        self.ctx.check("swg_ensemble_kick_variant", self.ctx.lib.swg_ensemble_kick_variant(self.h, 5, C.byref(v)))
        return int(v.value)

    def kick_warps(self) -> int:
        """Warps per block of the symmetric pl-pl kick in use (-1 before the first mixed kick)."""
        v = C.c_int(-1)
        self.ctx.check("swg_ensemble_kick_variant", self.ctx.lib.swg_ensemble_kick_variant(self.h, 3, C.byref(v)))
        return int(v.value)

    def getacch_int_pl(self):
        """Pair accelerations of every system's massive bodies from the current positions."""
        out = np.zeros((int(self.poff[-1]), 3))
        self.ctx.check("swg_ensemble_getacch_int_pl", self.ctx.lib.swg_ensemble_getacch_int_pl(self.h, _ptr(out)))
        return out

    def kick_variant(self):
        """Kernels in use by the mixed pl-pl and pl-tp kicks: a broadcast tile shape,
        SWG_KICK_SYMMETRIC, or -1 before the first mixed kick of that kind."""
        out = []
        for kind in (0, 1):
            v = C.c_int(-1)
            self.ctx.check("swg_ensemble_kick_variant", self.ctx.lib.swg_ensemble_kick_variant(self.h, kind, C.byref(v)))
            out.append(int(v.value))
        return {"pl": out[0], "tp": out[1]}

    def profile(self, enable: bool = True):
        self.ctx.check("swg_ensemble_profile", self.ctx.lib.swg_ensemble_profile(self.h, int(bool(enable))))

    def profile_read(self):
        out = np.zeros(10)
        self.ctx.check("swg_ensemble_profile_read", self.ctx.lib.swg_ensemble_profile_read(self.h, _ptr(out)))
        return {k: {"launches": int(out[2 * i]), "ms": float(out[2 * i + 1])}
                for i, k in enumerate(self.PROFILE_CLASSES)}

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.ctx.lib.swg_ensemble_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
