"""GPU parity of the kernel-level C ABI against the CPU oracle.

FP64 kick, drift and encounter lists must be bit-identical to the oracle (the
serial reference loop without FMA contraction).  The mixed-precision kick is
checked against the FP64 oracle with the tolerance stated in each test.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import SWG_ENC_SORTSWEEP, SWG_ENC_TRIANGULAR, SWG_FP64, SWG_MIXED
from swiftest_gb300 import initial_conditions as IC

pytestmark = pytest.mark.gpu


def _sys(seed, npl, ntp, **kw):
    cb, pl, tp = IC.make_system(seed=seed, npl=npl, ntp=ntp, **kw)
    return cb, IC.sort_for_integrator(pl, "SYMBA"), tp


# ---------------------------------------------------------------- kick
@pytest.mark.parametrize("npl", [1, 2, 7, 128, 129, 1000])
@pytest.mark.parametrize("rad", [False, True])
def test_kick_tri_fp64_bitexact(ctx, npl, rad):
    cb, pl, _ = _sys(npl, npl, 0)
    R = pl["radius"] * (50.0 if rad else 1.0) if rad else None
    acc0 = np.random.default_rng(npl).normal(size=(npl, 3)) * 1e-3
    g = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], R, acc=acc0, precision=SWG_FP64)
    r = O.kick_tri_pl(pl["rh"], pl["Gmass"], R, acc=acc0)
    assert np.array_equal(g, r)


@pytest.mark.parametrize("npl,nplm", [(300, 100), (300, 200), (257, 1), (64, 64)])
def test_kick_tri_gmtiny_bitexact(ctx, npl, nplm):
    cb, pl, _ = _sys(5, npl, 0)
    g = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], nplm=nplm)
    r = O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], nplm=nplm)
    assert np.array_equal(g, r)


@pytest.mark.parametrize("npl,nplm", [(200, 200), (200, 50)])
def test_kick_flat_bitexact(ctx, npl, nplm):
    cb, pl, _ = _sys(6, npl, 0)
    # canonical list derived on the GPU from tile coordinates
    g = ctx.kick_getacch_int_all_flat_pl(pl["rh"], pl["Gmass"], pl["radius"], nplm=nplm)
    r = O.kick_flat_pl(pl["rh"], pl["Gmass"], pl["radius"], nplm=nplm)
    assert np.array_equal(g, r)
    # explicit pair list (serial list-order kernel)
    k = O.flatten(npl, nplm)
    g2 = ctx.kick_getacch_int_all_flat_pl(pl["rh"], pl["Gmass"], pl["radius"], k_plpl=k, nplm=nplm)
    assert np.array_equal(g2, r)


@pytest.mark.parametrize("ntp,npl", [(1, 1), (1000, 100), (129, 300)])
def test_kick_tp_bitexact(ctx, ntp, npl):
    cb, pl, tp = _sys(7, npl, ntp)
    m = (np.arange(ntp) % 3 != 1).astype(np.int32)
    g = ctx.kick_getacch_int_all_tp(tp["rh"], pl["rh"], pl["Gmass"], lmask=m)
    r = O.kick_tp(tp["rh"], pl["rh"], pl["Gmass"], lmask=m)
    assert np.array_equal(g, r)


def _relerr(a, b):
    # per-body error relative to the body's acceleration magnitude
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


@pytest.mark.parametrize("npl", [64, 1000, 4096, 16384])  # 16384: the symmetric kernel
def test_kick_mixed_plpl_tolerance(ctx, npl):
    cb, pl, _ = _sys(8, npl, 0)
    g = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], precision=SWG_MIXED)
    r = O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"])
    e = _relerr(g, r)
    # FP32 pair terms with float-float partial sums: 2e-5 max, 1e-6 RMS per body
    assert e.max() < 2e-5, e.max()
    assert np.sqrt(np.mean(e ** 2)) < 1e-6


@pytest.mark.parametrize("ntp,npl", [(5000, 500), (100, 2000)])
def test_kick_mixed_tp_tolerance(ctx, ntp, npl):
    cb, pl, tp = _sys(9, npl, ntp)
    g = ctx.kick_getacch_int_all_tp(tp["rh"], pl["rh"], pl["Gmass"], precision=SWG_MIXED)
    r = O.kick_tp(tp["rh"], pl["rh"], pl["Gmass"])
    e = _relerr(g, r)
    assert e.max() < 2e-5, e.max()
    assert np.sqrt(np.mean(e ** 2)) < 1e-6


@pytest.mark.parametrize("npl", [1000, 16000])  # broadcast kernel, symmetric kernel
@pytest.mark.parametrize("guard", ["radius", "index"])
def test_kick_mixed_close_and_overlapping_pairs(ctx, guard, npl):
    # bodies placed next to others: pairs within the sum of the radii are dropped by the
    # radius rule, a close pair just outside it is kept and dominates.  Pairs across tiles,
    # within one 128-body tile across 32-body sub-tiles (10, 100) and within one sub-tile
    # (40, 45)
    cb, pl, _ = _sys(12, npl, 0)
    rh, R = pl["rh"].copy(), pl["radius"].copy()
    u = np.array([0.6, -0.48, 0.64])
    f = npl // 1000
    pairs = [(5, 700 * f, 1e-6), (300 * f, 950 * f, 1e-6), (513 * f, 2, 3e-6), (140 * f, 260 * f, 1e-4),
             (10, 100, 2e-6), (40, 45, 2e-6)]
    for i, j, sep in pairs:
        rh[j] = rh[i] + sep * u
        R[i] = R[j] = 1e-5
    Rk = R if guard == "radius" else None
    g = ctx.kick_getacch_int_all_tri_pl(rh, pl["Gmass"], Rk, precision=SWG_MIXED)
    r = O.kick_tri_pl(rh, pl["Gmass"], Rk)
    e = _relerr(g, r)
    assert np.all(np.isfinite(g))
    if guard == "radius":
        assert e.max() < 2e-5, e.max()
    else:  # without the radius rule the 1e-6 pairs are kept: FP32 r^-3 of a 1e-6 separation
        keep = np.ones(len(e), bool)
        keep[[b for i, j, sep in pairs if sep < 1e-5 for b in (i, j)]] = False
        assert e[keep].max() < 2e-5, e[keep].max()
        assert e[~keep].max() < 1e-3, e[~keep].max()


def test_kick_mixed_deterministic(ctx):
    cb, pl, tp = _sys(10, 3000, 0)
    a = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], precision=SWG_MIXED)
    b = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], precision=SWG_MIXED)
    assert np.array_equal(a, b)


def test_kick_newton_third_law(ctx):
    cb, pl, _ = _sys(11, 500, 0)
    a = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], None)
    p = (pl["Gmass"][:, None] * a).sum(axis=0)
    scale = (pl["Gmass"][:, None] * np.abs(a)).sum(axis=0)
    assert np.all(np.abs(p) < 1e-13 * scale)


# ---------------------------------------------------------------- drift
def test_drift_bitexact_elliptic(ctx):
    # kepmd and Newton paths with the series initial guess use only +-*/ and sqrt:
    # bit-identical to the oracle
    cb, pl, tp = _sys(12, 500, 3000, sig_e=0.3)
    x = np.concatenate([pl["rh"], tp["rh"]])
    v = np.concatenate([pl["vh"], tp["vh"]])
    mu = np.full(len(x), IC.GMCB)
    m = np.ones(len(x), np.int32)
    m[::17] = 0
    gx, gv, gf = ctx.drift_all(mu, x, v, 0.005, lmask=m)
    rx, rv, rf = O.drift_all(mu, x, v, 0.005, lmask=m)
    assert np.array_equal(gf, rf)
    assert np.array_equal(gx, rx) and np.array_equal(gv, rv)


@pytest.mark.parametrize("dt", [0.005, 0.5, 7.3])
def test_drift_general(ctx, dt):
    # hyperbolic (cube-root initial guess) and long steps (sine initial guess) call
    # libm pow/sin, whose last bit may differ between CUDA and glibc: 1e-10 relative
    cb, pl, tp = _sys(14, 500, 3000, sig_e=0.3)
    x = np.concatenate([pl["rh"], tp["rh"]])
    v = np.concatenate([pl["vh"], tp["vh"]])
    v[:50] *= 1.6
    v[50:60] *= np.sqrt(2.0)
    mu = np.full(len(x), IC.GMCB)
    gx, gv, gf = ctx.drift_all(mu, x, v, dt)
    rx, rv, rf = O.drift_all(mu, x, v, dt)
    assert np.array_equal(gf, rf)
    ok = gf == 0
    ex = np.linalg.norm(gx - rx, axis=1) / np.linalg.norm(rx, axis=1)
    ev = np.linalg.norm(gv - rv, axis=1) / np.linalg.norm(rv, axis=1)
    assert ex[ok].max() < 1e-10 and ev[ok].max() < 1e-10


def test_drift_gr_bitexact(ctx):
    cb, pl, tp = _sys(13, 100, 100)
    x, v = tp["rh"], tp["vh"]
    inv_c2 = 1.0 / (63241.077 ** 2)
    gx, gv, gf = ctx.drift_all(IC.GMCB, x, v, 0.01, lgr=True, inv_c2=inv_c2)
    rx, rv, rf = O.drift_all(IC.GMCB, x, v, 0.01, lgr=True, inv_c2=inv_c2)
    assert np.array_equal(gx, rx) and np.array_equal(gv, rv)


# ---------------------------------------------------------------- encounters
def _dense(seed, n, ntp=0, spread=0.02):
    rng = np.random.default_rng(seed)
    r = rng.normal(size=(n, 3)) * spread + np.array([1.0, 0, 0])
    v = rng.normal(size=(n, 3)) * 0.05 + np.array([0, 6.28, 0])
    renc = np.exp(rng.uniform(np.log(2e-4), np.log(4e-3), n))
    rt = rng.normal(size=(ntp, 3)) * spread + np.array([1.0, 0, 0])
    vt = rng.normal(size=(ntp, 3)) * 0.05 + np.array([0, 6.28, 0])
    return r, v, renc, rt, vt


@pytest.mark.parametrize("mode", [SWG_ENC_TRIANGULAR, SWG_ENC_SORTSWEEP])
@pytest.mark.parametrize("n", [0, 1, 2, 300, 3000])
def test_encounter_plpl_bitexact(ctx, mode, n):
    r, v, renc, _, _ = _dense(n, n)
    g = ctx.encounter_check_all_plpl(r, v, renc, 0.01, mode=mode, cap=4)
    o = O.encounter_plpl(r, v, renc, 0.01, mode=mode)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)
    if n >= 300:
        assert len(g[0]) > 0


@pytest.mark.parametrize("mode", [SWG_ENC_TRIANGULAR, SWG_ENC_SORTSWEEP])
def test_encounter_pltp_bitexact(ctx, mode):
    r, v, renc, rt, vt = _dense(21, 400, 5000)
    g = ctx.encounter_check_all_pltp(r, v, rt, vt, renc, 0.01, mode=mode, cap=8)
    o = O.encounter_pltp(r, v, rt, vt, renc, 0.01, mode=mode)
    assert len(o[0]) > 0
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", [SWG_ENC_TRIANGULAR, SWG_ENC_SORTSWEEP])
def test_encounter_plplm_bitexact(ctx, mode):
    r, v, renc, _, _ = _dense(22, 600)
    nplm = 150
    g = ctx.encounter_check_all_plplm(r[:nplm], v[:nplm], r[nplm:], v[nplm:], renc[:nplm], renc[nplm:], 0.01,
                                      mode=mode)
    o = O.encounter_plplm(r[:nplm], v[:nplm], r[nplm:], v[nplm:], renc[:nplm], renc[nplm:], 0.01, mode=mode)
    assert len(o[0]) > 0
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


def test_encounter_triangular_large_sparse(ctx):
    # disk-like geometry: the FP32 prefilter rejects almost every pair
    cb, pl, tp = _sys(23, 2000, 10000, amin=0.3, amax=3.0)
    renc = pl["rhill"] * 3.0
    g = ctx.encounter_check_all_pltp(pl["rh"], pl["vh"], tp["rh"], tp["vh"], renc, 0.005)
    o = O.encounter_pltp(pl["rh"], pl["vh"], tp["rh"], tp["vh"], renc, 0.005)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)
    g = ctx.encounter_check_all_plpl(pl["rh"], pl["vh"], renc, 0.005)
    o = O.encounter_plpl(pl["rh"], pl["vh"], renc, 0.005)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


def test_encounter_boundary_cases(ctx):
    # pairs placed exactly at, just inside and just outside the encounter radius
    R = 1e-3
    base = np.array([1.0, 0.0, 0.0])
    offs = [R * (1 - 1e-12), R, R * (1 + 1e-12), 0.5 * R, 2 * R]
    r, v = [], []
    for k, d in enumerate(offs):
        c = base + np.array([0.0, 0.1 * k, 0.0])
        r += [c, c + np.array([d, 0.0, 0.0])]
        v += [np.zeros(3), np.array([0.0, 1e-3, 0.0])]
    r, v = np.array(r), np.array(v)
    renc = np.full(len(r), R / 2)
    g = ctx.encounter_check_all_plpl(r, v, renc, 0.001)
    o = O.encounter_plpl(r, v, renc, 0.001)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


# ---------------------------------------------------------------- orbital elements
@pytest.mark.parametrize("emin,emax", [(0.0, 0.18), (0.18, 0.8), (0.8, 0.99), (1.01, 1.5), (1.5, 8.0)])
def test_orbel_matches_oracle(ctx, emin, emax):
    # el2xv over every Kepler-solver branch and xv2el of the results, against the oracle;
    # CUDA's and glibc's sin/cos/sinh/log/pow/acos/atan2 may differ in the last bit: 1e-11
    rng = np.random.default_rng(int(emin * 100) + 1)
    n = 4000
    a, e = rng.uniform(0.3, 30.0, n), rng.uniform(emin, emax, n)
    inc, capom, omega = rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n)
    capm = rng.uniform(-20.0, 20.0, n) if emin > 1.0 else rng.uniform(-3.0, 3.0, n)
    mu = IC.GMCB * (1.0 + rng.uniform(0.0, 1e-6, n))
    g_rh, g_vh = ctx.el2xv(mu, a, e, inc, capom, omega, capm)
    r_rh, r_vh = O.el2xv(mu, a, e, inc, capom, omega, capm)
    for g, r in ((g_rh, r_rh), (g_vh, r_vh)):
        rel = np.linalg.norm(g - r, axis=1) / np.linalg.norm(r, axis=1)
        assert rel.max() < 1e-11, rel.max()
    ge, re = ctx.xv2el(mu, r_rh, r_vh), O.xv2el(mu, r_rh, r_vh)
    for k in ("a", "e"):
        np.testing.assert_allclose(ge[k], re[k], rtol=1e-11, atol=1e-13)
    for k in ("inc", "capom", "omega", "capm", "varpi", "lam", "f", "cape", "capf"):
        d = np.abs(np.angle(np.exp(1j * (ge[k] - re[k])))) if k != "capm" or emax <= 1.0 else np.abs(ge[k] - re[k])
        assert d.max() < 1e-9, (k, d.max())
