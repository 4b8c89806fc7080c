"""The radix sort under the sort-and-sweep encounter check, and sort-and-sweep in ensembles.

* swg_util_sort_index (util_sort with an index, base_module.f90:1361-1472) against numpy's
  stable argsort: tile-boundary sizes, ties, negative values, -0.0 against +0.0 (equal),
  constant arrays (every pass skipped) and a million values.
* SyMBA ensembles with SORTSWEEP level-0 checks (encounter_check.f90:143-326, 763-988): each
  system's trajectory, lists and statistics are the oracle's for that system stepped alone in
  the same modes, bit for bit, for every combination of the pl-pl and pl-tp modes.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import Ensemble

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 3, 2047, 2048, 2049, 6000, 1_000_000])
def test_sort_index_matches_stable_argsort(ctx, n):
    rng = np.random.default_rng(n)
    a = rng.normal(size=n) * 10.0 ** rng.integers(-3, 4, size=n)
    a[rng.integers(0, n, size=n // 3)] = 1.25  # ties
    if n > 3:
        a[:4] = [0.0, -0.0, -1.0, 0.0]
    got = ctx.util_sort_index(a)
    assert np.array_equal(got, np.argsort(a, kind="stable") + 1)


def test_sort_index_constant_and_integer_keys(ctx):
    a = np.full(5000, 3.5)
    assert np.array_equal(ctx.util_sort_index(a), np.arange(1, 5001))
    b = np.random.default_rng(1).integers(0, 7, size=10000).astype(np.float64)
    assert np.array_equal(ctx.util_sort_index(b), np.argsort(b, kind="stable") + 1)


def _disk_ensemble(seeds, npl=150, ntp=200):
    systems = []
    for seed in seeds:
        cb, pl, tp = IC.make_system(seed=seed, npl=npl, ntp=ntp, amin=0.8, amax=1.3, mmin=1e-9, mmax=1e-6)
        systems.append((IC.sort_for_integrator(pl, "SYMBA"), tp))
    k = len(systems)
    return {"integrator": "SYMBA", "dt": 0.005, "rhscale": 3.0,
            "npl": np.array([len(p["Gmass"]) for p, _ in systems], np.int32),
            "ntp": np.array([len(t["rh"]) for _, t in systems], np.int32),
            "GMcb": np.full(k, IC.GMCB), "Rcb": np.full(k, IC.RCB),
            "pl": {f: np.concatenate([p[f] for p, _ in systems]) for f in ("rh", "vh", "Gmass", "radius", "rhill")},
            "tp": {f: np.concatenate([t[f] for _, t in systems]) for f in ("rh", "vh")}, "systems": systems}


@pytest.mark.parametrize("modes", [("SORTSWEEP", "SORTSWEEP"), ("SORTSWEEP", "TRIANGULAR"),
                                   ("TRIANGULAR", "SORTSWEEP")])
def test_ensemble_sortsweep_bitexact(ctx, modes):
    E = _disk_ensemble((41, 42, 43))
    ens = Ensemble(ctx, E, precision="FP64", encounter_check_plpl=modes[0], encounter_check_pltp=modes[1])
    cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
    refs = [O.OracleSystem("SYMBA", cb, pl, tp, dt=E["dt"], rhscale=E["rhscale"], encounter_check_plpl=modes[0],
                           encounter_check_pltp=modes[1]) for pl, tp in E["systems"]]
    npairs = 0
    for _ in range(4):
        ens.step(25)
        for r in refs:
            r.step(25)
        for s, r in enumerate(refs):
            gi = ens.plpl_list(s)
            ri = r.plpl_list()
            assert all(np.array_equal(a, b) for a, b in zip(gi, ri)), s
            npairs += len(ri[0])
    assert npairs > 0
    rh, vh, st = ens.get_pl()
    trh, tvh, tst = ens.get_tp()
    for s, r in enumerate(refs):
        a, b = ens.poff[s], ens.poff[s + 1]
        orh, ovh, ost = r.get_pl()
        assert np.array_equal(rh[a:b], orh) and np.array_equal(vh[a:b], ovh) and np.array_equal(st[a:b], ost), s
        a, b = ens.toff[s], ens.toff[s + 1]
        orh, ovh, ost = r.get_tp()
        assert np.array_equal(trh[a:b], orh) and np.array_equal(tvh[a:b], ovh) and np.array_equal(tst[a:b], ost), s
    tot = {k: sum(r.stats()[k] for r in refs) for k in ("plpl_encounters", "pltp_encounters", "collisions")}
    es = ens.stats()
    assert all(es[k] == v for k, v in tot.items()), (es, tot)
    ens.close()
