"""The SyMBA recursion on both of its memory forms (symba_step_recur_system,
symba_step.f90:163-262).

The recursion kernel copies the listed bodies and the list entries into shared memory when
they fit (up to 160 KB for a single system, 64 KB per system in an ensemble launch) and
works on the global arrays otherwise; both forms take the same arithmetic in the same
order.  The other SyMBA tests run the shared-memory form (their lists are short); here a
narrow ring with 10-Hill-radius encounter spheres gives ~750 pl-pl and ~500 pl-tp level-0
pairs, whose stage (~265 KB) does not fit, so the recursion runs on the global arrays:
single system, and an ensemble where that system sits beside two that are staged.  Every
system must stay the oracle's, bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import Ensemble, NBodySystem

pytestmark = pytest.mark.gpu

KW = dict(dt=0.002, rhscale=10.0)


def _ring(seed):
    cb, pl, tp = IC.make_system(seed=seed, npl=300, ntp=300, amin=0.95, amax=1.05, mmin=1e-8, mmax=1e-6)
    return cb, IC.sort_for_integrator(pl, "SYMBA"), tp


def _disk(seed):
    cb, pl, tp = IC.make_system(seed=seed, npl=150, ntp=200, amin=0.8, amax=1.3, mmin=1e-9, mmax=1e-6)
    return cb, IC.sort_for_integrator(pl, "SYMBA"), tp


def _same(gpu_state, ref_state):
    return all(np.array_equal(a, b) for a, b in zip(gpu_state, ref_state))


def test_large_lists_single_system(ctx):
    cb, pl, tp = _ring(5)
    gpu = NBodySystem(ctx, "SYMBA", cb, pl, tp, **KW)
    ref = O.OracleSystem("SYMBA", cb, pl, tp, **KW)
    for _ in range(4):
        gpu.step(5)
        ref.step(5)
        assert len(ref.plpl_list()[0]) > 600  # beyond the shared-memory stage
        assert _same(gpu.plpl_list(), ref.plpl_list()) and _same(gpu.pltp_list(), ref.pltp_list())
    assert _same(gpu.get_pl(), ref.get_pl()) and _same(gpu.get_tp(), ref.get_tp())
    assert gpu.stats() == ref.stats()
    gpu.close()


def test_large_and_small_lists_in_one_ensemble(ctx):
    parts = [_disk(41), _ring(5), _disk(43)]
    systems = [(pl, tp) for _, pl, tp in parts]
    k = len(systems)
    E = {"integrator": "SYMBA", **KW,
         "npl": np.array([len(p["Gmass"]) for p, _ in systems], np.int32),
         "ntp": np.array([len(t["rh"]) for _, t in systems], np.int32),
         "GMcb": np.full(k, IC.GMCB), "Rcb": np.full(k, IC.RCB),
         "pl": {f: np.concatenate([p[f] for p, _ in systems]) for f in ("rh", "vh", "Gmass", "radius", "rhill")},
         "tp": {f: np.concatenate([t[f] for _, t in systems]) for f in ("rh", "vh")}, "systems": systems}
    ens = Ensemble(ctx, E, precision="FP64")
    cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
    refs = [O.OracleSystem("SYMBA", cb, pl, tp, **KW) for pl, tp in systems]
    for _ in range(3):
        ens.step(5)
        for r in refs:
            r.step(5)
        for s, r in enumerate(refs):
            assert _same(ens.plpl_list(s), r.plpl_list()), s
    rh, vh, st = ens.get_pl()
    trh, tvh, tst = ens.get_tp()
    for s, r in enumerate(refs):
        a, b = ens.poff[s], ens.poff[s + 1]
        assert _same((rh[a:b], vh[a:b], st[a:b]), r.get_pl()), s
        a, b = ens.toff[s], ens.toff[s + 1]
        assert _same((trh[a:b], tvh[a:b], tst[a:b]), r.get_tp()), s
    assert len(refs[1].plpl_list()[0]) > 600 and 0 < len(refs[0].plpl_list()[0]) < 100
    ens.close()
