"""Parity at the benchmark configurations' own sizes (the other GPU tests use reduced ones).

* C2 (kick only, m in [1e-12, 1e-8] Msun, a in [0.5, 5] AU): the FP64 pl-pl and pl-tp kicks
  at N = 16,384 pl and 4N tp are the oracle's bits; the mixed kicks at N = 65,536 (the
  symmetric pl-pl kernel; the pl-tp kick on 4N tp, checked on every 16th tp) are within the
  mixed-kick tolerance, 2e-5 per body relative to |a|.
* C0 (HELIO, 100 pl + 1000 tp, dt 0.01 yr): the full 1000 steps, bit for bit.
* C1 (SyMBA, 2000 pl + 10,000 tp, 1-Hill-radius encounter radius, dt 0.005 yr): 50 steps,
  with the level-0 pl-pl and pl-tp encounter lists compared every 10 steps, bit for bit.
* C4 (256 SyMBA disks, 547,900 pl): one FP64 step of the whole batched ensemble, every
  system compared with the oracle stepping it alone.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import SWG_FP64, SWG_MIXED
from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import Ensemble, NBodySystem

pytestmark = pytest.mark.gpu

MIXED_TOL = 2e-5


def _relerr(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def _c2(n):
    cb, pl, tp = IC.make_system(seed=2, npl=n, ntp=4 * n, mmin=1e-12, mmax=1e-8, amin=0.5, amax=5.0)
    return IC.sort_for_integrator(pl, "SYMBA"), tp


def test_c2_fp64_kick_bitexact_16k(ctx):
    pl, tp = _c2(16384)
    g = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], precision=SWG_FP64)
    assert np.array_equal(g, O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"]))
    g = ctx.kick_getacch_int_all_tp(tp["rh"], pl["rh"], pl["Gmass"], precision=SWG_FP64)
    assert np.array_equal(g, O.kick_tp(tp["rh"], pl["rh"], pl["Gmass"]))


def test_c2_mixed_kick_tolerance_64k(ctx):
    pl, tp = _c2(65536)
    g = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], precision=SWG_MIXED)
    r = O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"])
    assert _relerr(g, r).max() < MIXED_TOL
    g = ctx.kick_getacch_int_all_tp(tp["rh"], pl["rh"], pl["Gmass"], precision=SWG_MIXED)
    sub = np.arange(0, len(tp["rh"]), 16)  # tp accelerations are independent of each other
    r = O.kick_tp(tp["rh"][sub], pl["rh"], pl["Gmass"])
    assert _relerr(g[sub], r).max() < MIXED_TOL


def _config_system(name):
    c = IC.CONFIGS[name]
    cb, pl, tp = IC.make_system(seed=c["seed"], npl=c["npl"], ntp=c["ntp"], mmin=c["mmin"], mmax=c["mmax"],
                                amin=c["amin"], amax=c["amax"], sig_e=c["sig_e"], sig_i=c["sig_i"])
    return c, cb, IC.sort_for_integrator(pl, c["integrator"]), tp


def _same_state(gpu, ref):
    for a, b in zip(gpu.get_pl() + gpu.get_tp(), ref.get_pl() + ref.get_tp()):
        assert np.array_equal(a, b)


def test_c0_helio_1000_steps_bitexact(ctx):
    c, cb, pl, tp = _config_system("C0")
    gpu = NBodySystem(ctx, "HELIO", cb, pl, tp, dt=c["dt"], precision="FP64")
    ref = O.OracleSystem("HELIO", cb, pl, tp, dt=c["dt"])
    gpu.step(c["nsteps"])
    ref.step(c["nsteps"])
    _same_state(gpu, ref)
    gpu.close()


def test_c1_symba_50_steps_lists_bitexact(ctx):
    c, cb, pl, tp = _config_system("C1")
    kw = dict(dt=c["dt"], rhscale=c["rhscale"])
    gpu = NBodySystem(ctx, "SYMBA", cb, pl, tp, precision="FP64", **kw)
    ref = O.OracleSystem("SYMBA", cb, pl, tp, **kw)
    npp = npt = 0
    for _ in range(5):
        gpu.step(10)
        ref.step(10)
        for g, r in ((gpu.plpl_list(), ref.plpl_list()), (gpu.pltp_list(), ref.pltp_list())):
            assert all(np.array_equal(a, b) for a, b in zip(g, r))
        npp += len(ref.plpl_list()[0])
        npt += len(ref.pltp_list()[0])
    assert npp > 0 and npt > 0
    _same_state(gpu, ref)
    assert gpu.stats() == ref.stats()
    gpu.close()


def test_c4_full_ensemble_step_fp64(ctx):
    E = IC.make_ensemble("C4")
    assert len(E["npl"]) == 256
    ens = Ensemble(ctx, E, precision="FP64")
    ens.step(1)
    rh, vh, st = ens.get_pl()
    cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
    for s, (pl, tp) in enumerate(E["systems"]):
        ref = O.OracleSystem("SYMBA", cb, pl, tp, dt=E["dt"], rhscale=E["rhscale"], lclose=True)
        ref.step(1)
        orh, ovh, ost = ref.get_pl()
        a, b = ens.poff[s], ens.poff[s + 1]
        assert np.array_equal(rh[a:b], orh) and np.array_equal(vh[a:b], ovh) and np.array_equal(st[a:b], ost), s
    ens.close()
