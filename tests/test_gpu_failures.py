"""The reference's failure behaviours on the GPU path, with the failing inputs made on the host.

* Danby drift failure: a body 1e-8 AU from the central body moving at 1e5 AU/yr defeats the
  universal-variable solver (iflag 2, swiftest_drift.f90:111-138), deterministically and
  without NaNs.  The kernel-level iflag, HELIO and SyMBA's DISCARDED_DRIFTERR status
  (helio_drift.f90:41-49, symba_drift.f90) and WHM's abort (whm_drift.f90:38-54, here the
  status SWG_ERR_DRIFT from the step call, single system and ensemble) are checked against
  the oracle.
* The caller-capacity protocol of the encounter lists (mirroring encounter_util_resize_list,
  encounter_util.f90:294-329): a call whose list does not fit returns SWG_ERR_CAPACITY with
  the required size, and the retry with that capacity returns the full list.
The SyMBA recursion-underflow error (symba_step.f90:196-201) needs 33 recursion levels; the
sub-steps double and more per level, so no test can reach it in bounded time.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import _lib as L
from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import Ensemble, NBodySystem

pytestmark = pytest.mark.gpu

BAD_R, BAD_V = [1e-8, 0.0, 0.0], [0.0, 1e5, 3.0]  # the state that defeats the Danby solver


def _system(integrator, k=5, tp_k=4, seed=3):
    cb, pl, tp = IC.make_system(seed=seed, npl=20, ntp=30, amin=0.5, amax=2.0)
    pl = IC.sort_for_integrator(pl, integrator)
    pl["rh"][k], pl["vh"][k] = BAD_R, BAD_V
    tp["rh"][tp_k], tp["vh"][tp_k] = BAD_R, BAD_V
    return cb, pl, tp


def test_drift_failure_flag(ctx):
    mu = np.full(3, IC.GMCB)
    x = np.array([[1.0, 0.0, 0.0], BAD_R, [0.0, 1.5, 0.0]])
    v = np.array([[0.0, 6.28, 0.0], BAD_V, [-5.1, 0.0, 0.1]])
    xg, vg, fg = ctx.drift_all(mu, x, v, 0.01)
    xo, vo, fo = O.drift_all(mu, x.copy(), v.copy(), 0.01)
    assert list(fo) == [0, 2, 0]
    assert np.array_equal(fg, fo)
    assert np.array_equal(xg[[0, 2]], xo[[0, 2]]) and np.array_equal(vg[[0, 2]], vo[[0, 2]])


@pytest.mark.parametrize("integrator", ["HELIO", "SYMBA"])
def test_drift_failure_discards_body(ctx, integrator):
    cb, pl, tp = _system(integrator)
    kw = dict(dt=0.01, rhscale=1.0)
    gpu = NBodySystem(ctx, integrator, cb, pl, tp, precision="FP64", **kw)
    ref = O.OracleSystem(integrator, cb, pl, tp, **kw)
    gpu.step(3)
    ref.step(3)
    g, r = gpu.get_pl(), ref.get_pl()
    assert r[2][5] == -7  # DISCARDED_DRIFTERR
    assert np.array_equal(g[2], r[2]) and np.array_equal(gpu.get_tp()[2], ref.get_tp()[2])
    ok = r[2] == 0  # the bodies that drifted normally are the oracle's, bit for bit
    assert np.array_equal(g[0][ok], r[0][ok]) and np.array_equal(g[1][ok], r[1][ok])
    gpu.close()


def test_whm_drift_failure_stops_the_run(ctx):
    cb, pl, tp = _system("WHM", k=0)
    with pytest.raises(RuntimeError, match="-5"):
        O.OracleSystem("WHM", cb, pl, tp, dt=0.01).step(1)
    gpu = NBodySystem(ctx, "WHM", cb, pl, tp, dt=0.01, precision="FP64")
    with pytest.raises(L.SwiftestGB300Error) as ei:
        gpu.step(1)
    assert ei.value.code == L.SWG_ERR_DRIFT
    gpu.close()


def test_whm_ensemble_drift_failure_stops_the_run(ctx):
    systems = []
    for seed, bad in ((3, False), (4, True), (5, False)):
        cb, pl, tp = IC.make_system(seed=seed, npl=20, ntp=30, amin=0.5, amax=2.0)
        pl = IC.sort_for_integrator(pl, "WHM")
        if bad:
            pl["rh"][0], pl["vh"][0] = BAD_R, BAD_V
        systems.append((pl, tp))
    E = {"integrator": "WHM", "dt": 0.01, "rhscale": 6.5,
         "npl": np.array([len(p["Gmass"]) for p, _ in systems], np.int32),
         "ntp": np.array([len(t["rh"]) for _, t in systems], np.int32),
         "GMcb": np.full(3, IC.GMCB), "Rcb": np.full(3, IC.RCB),
         "pl": {k: np.concatenate([p[k] for p, _ in systems]) for k in ("rh", "vh", "Gmass", "radius", "rhill")},
         "tp": {k: np.concatenate([t[k] for _, t in systems]) for k in ("rh", "vh")}, "systems": systems}
    for prec in ("FP64", "MIXED"):
        ens = Ensemble(ctx, E, precision=prec)
        with pytest.raises(L.SwiftestGB300Error) as ei:
            ens.step(1)
        assert ei.value.code == L.SWG_ERR_DRIFT
        ens.close()


@pytest.mark.parametrize("mode", [L.SWG_ENC_TRIANGULAR, L.SWG_ENC_SORTSWEEP])
def test_encounter_capacity_protocol(ctx, mode):
    cb, pl, _ = IC.make_system(seed=21, npl=400, ntp=0, amin=0.8, amax=1.2)
    r, v = np.ascontiguousarray(pl["rh"]), np.ascontiguousarray(pl["vh"])
    renc = np.ascontiguousarray(pl["rhill"] * 20.0)
    lib, h = ctx.lib, ctx.h
    n = ctypes.c_int64(0)
    buf = [np.zeros(1, np.int32) for _ in range(3)]
    p = [b.ctypes.data_as(ctypes.c_void_p) for b in buf]
    args = (mode, 400, r.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p),
            renc.ctypes.data_as(ctypes.c_void_p), 0.01)
    rc = lib.swg_encounter_check_all_plpl(h, *args, 1, ctypes.byref(n), *p, L.SWG_MEM_HOST)
    assert rc == L.SWG_ERR_CAPACITY and n.value > 1
    need = n.value
    buf = [np.zeros(need, np.int32) for _ in range(3)]
    p = [b.ctypes.data_as(ctypes.c_void_p) for b in buf]
    rc = lib.swg_encounter_check_all_plpl(h, *args, need, ctypes.byref(n), *p, L.SWG_MEM_HOST)
    assert rc == L.SWG_OK and n.value == need
    o1, o2, _ = O.encounter_plpl(r, v, renc, 0.01, mode=mode)
    assert np.array_equal(buf[0], o1) and np.array_equal(buf[1], o2)
