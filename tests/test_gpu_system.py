"""GPU parity of the device-resident step loops (WHM, HELIO, SyMBA) against the oracle.

In FP64 mode the device path evaluates every expression of the serial
reference loop in the same order, so trajectories must match the oracle bit
for bit; the stated tolerance (1e-9 relative after the run) is asserted as
well for the record.  The mixed path is checked for energy and
angular-momentum conservation against the FP64 path.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import NBodySystem

pytestmark = pytest.mark.gpu


def _setup(integ, seed, npl, ntp, **kw):
    cb, pl, tp = IC.make_system(seed=seed, npl=npl, ntp=ntp, **kw)
    return cb, IC.sort_for_integrator(pl, integ), tp


def _compare(gpu, ref, tol=1e-9):
    g_rh, g_vh, g_st = gpu.get_pl()
    r_rh, r_vh, r_st = ref.get_pl()
    t_rh, t_vh, t_st = gpu.get_tp()
    o_rh, o_vh, o_st = ref.get_tp()
    assert np.array_equal(g_st, r_st) and np.array_equal(t_st, o_st)
    for a, b in ((g_rh, r_rh), (g_vh, r_vh), (t_rh, o_rh), (t_vh, o_vh)):
        if len(a):
            rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
            assert rel.max() <= tol, rel.max()
    return (np.array_equal(g_rh, r_rh) and np.array_equal(g_vh, r_vh) and np.array_equal(t_rh, o_rh)
            and np.array_equal(t_vh, o_vh))


@pytest.mark.parametrize("integ", ["WHM", "HELIO"])
@pytest.mark.parametrize("loop", ["TRIANGULAR", "FLAT"])
def test_whm_helio_bitexact(ctx, integ, loop):
    cb, pl, tp = _setup(integ, 1, 100, 1000)
    kw = dict(dt=0.01, loop_mode=loop)
    gpu = NBodySystem(ctx, integ, cb, pl, tp, **kw)
    ref = O.OracleSystem(integ, cb, pl, tp, **kw)
    gpu.step(200)
    ref.step(200)
    assert _compare(gpu, ref)
    eg, er = gpu.energy(), ref.energy()
    assert abs(eg["te"] - er["te"]) <= 1e-12 * abs(er["te"])


@pytest.mark.parametrize("enc", ["TRIANGULAR", "SORTSWEEP"])
def test_symba_bitexact(ctx, enc):
    # compact disk with 3-Hill-radius encounter spheres: recursion exercised
    cb, pl, tp = _setup("SYMBA", 2, 200, 800, amin=0.8, amax=1.2, mmin=1e-9, mmax=1e-6)
    kw = dict(dt=0.005, rhscale=3.0, encounter_check_plpl=enc, encounter_check_pltp=enc)
    gpu = NBodySystem(ctx, "SYMBA", cb, pl, tp, **kw)
    ref = O.OracleSystem("SYMBA", cb, pl, tp, **kw)
    for _ in range(5):
        gpu.step(40)
        ref.step(40)
        gi = gpu.plpl_list()
        ri = ref.plpl_list()
        assert all(np.array_equal(a, b) for a, b in zip(gi, ri))
        gi = gpu.pltp_list()
        ri = ref.pltp_list()
        assert all(np.array_equal(a, b) for a, b in zip(gi, ri))
    assert _compare(gpu, ref)
    sg, sr = gpu.stats(), ref.stats()
    assert sg == sr
    assert sr["steps_with_encounters"] > 0 and sr["max_recursion"] >= 1


def test_symba_1000_steps_c1_shape(ctx):
    # C1-like disk (1-Hill-radius encounter radius), reduced body count
    cb, pl, tp = _setup("SYMBA", 0, 400, 2000, amin=0.3, amax=3.0)
    kw = dict(dt=0.005, rhscale=1.0)
    gpu = NBodySystem(ctx, "SYMBA", cb, pl, tp, **kw)
    ref = O.OracleSystem("SYMBA", cb, pl, tp, **kw)
    gpu.step(1000)
    ref.step(1000)
    assert _compare(gpu, ref, tol=1e-9)


def test_symba_mixed_conservation(ctx):
    cb, pl, tp = _setup("SYMBA", 4, 300, 0, amin=0.8, amax=1.5)
    kw = dict(dt=0.005, rhscale=2.0)
    f = NBodySystem(ctx, "SYMBA", cb, pl, None, precision="FP64", **kw)
    m = NBodySystem(ctx, "SYMBA", cb, pl, None, precision="MIXED", **kw)
    e0 = f.energy()
    f.step(500)
    m.step(500)
    ef, em = f.energy(), m.energy()
    dEf = abs(ef["te_helio"] - e0["te_helio"]) / abs(e0["te_helio"])
    dEm = abs(em["te_helio"] - e0["te_helio"]) / abs(e0["te_helio"])
    dLm = np.linalg.norm(em["L"] - e0["L"]) / np.linalg.norm(e0["L"])
    assert dEm < max(2 * dEf, 1e-9), (dEm, dEf)
    assert dLm < 1e-9


def test_context_close_releases_systems():
    # a system still open when its context closes is released by the context; closing it
    # afterwards is a no-op (no use of the freed context)
    from swiftest_gb300.api import Context
    c = Context(0)
    cb, pl, tp = _setup("SYMBA", 5, 50, 50)
    s = NBodySystem(c, "SYMBA", cb, pl, tp, dt=0.005, rhscale=3.0)
    s.step(2)
    c.close()
    s.close()
    assert s.h is None
