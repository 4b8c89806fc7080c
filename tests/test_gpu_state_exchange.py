"""The state exchange of an initialized system or ensemble (set_state / get_state_async).

A step after the first carries state of its own from the step before, as the reference's
steps do (HELIO: the barycentric velocities; WHM: the closing accelerations), so an upload
that changes the state reaches the next step only after reset_first_step (the reference's
lfirst flags).  With it the continued run equals, bit for bit in FP64, a run initialized
from the uploaded state; without it the step goes on from its own state.
"""
import numpy as np
import pytest

from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import Ensemble, NBodySystem

pytestmark = pytest.mark.gpu


def _modified(rh, vh):
    rh, vh = rh.copy(), vh.copy()
    vh[3] *= 1.001
    rh[5] += 1e-4
    return rh, vh


def _state(s):
    return s.get_pl()[:2] + s.get_tp()[:2]


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("integ", ["HELIO", "WHM"])
def test_system_set_state_reaches_step_after_reset(ctx, integ):
    cb, pl, tp = IC.make_system(seed=3, npl=60, ntp=200)
    pl = IC.sort_for_integrator(pl, integ)
    kw = dict(dt=0.01, lclose=False)
    runs = []
    for reset in (True, False):
        a = NBodySystem(ctx, integ, cb, pl, tp, **kw)
        a.step(10)
        rh, vh, _ = a.get_pl()
        trh, tvh, _ = a.get_tp()
        rh2, vh2 = _modified(rh, vh)
        a.set_state(rh2, vh2, trh, tvh)
        if reset:
            a.reset_first_step()
        a.step(10)
        runs.append(_state(a))
        a.close()
    fresh = NBodySystem(ctx, integ, cb, dict(pl, rh=rh2, vh=vh2), dict(tp, rh=trh, vh=tvh), **kw)
    fresh.step(10)
    want = _state(fresh)
    fresh.close()
    assert _same(runs[0], want)
    assert not _same(runs[1], want)


@pytest.mark.parametrize("integ", ["HELIO", "WHM"])
def test_ensemble_set_state_reaches_step_after_reset(ctx, integ):
    # the steps after the first replay from a CUDA graph; the reset drops it
    E = IC.make_ensemble("C3", nsys=3, scale=0.05, integrator=integ)
    kw = dict(precision="FP64", dt=0.01)
    a = Ensemble(ctx, E, **kw)
    a.step(10)
    rh, vh, _ = a.get_pl()
    trh, tvh, _ = a.get_tp()
    rh2, vh2 = _modified(rh, vh)
    a.set_state(rh2, vh2, trh, tvh)
    a.reset_first_step()
    a.step(10)
    got = _state(a)
    a.close()
    E2 = dict(E, pl=dict(E["pl"], rh=rh2, vh=vh2), tp=dict(E["tp"], rh=trh, vh=tvh))
    fresh = Ensemble(ctx, E2, **kw)
    fresh.step(10)
    assert _same(got, _state(fresh))
    fresh.close()
