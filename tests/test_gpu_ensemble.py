"""GPU parity of the batched ensemble (CSR-packed systems stepped together) against the oracle.

Every system of an ensemble must take exactly the steps it would take alone, so in
FP64 mode each system's state after the run is compared bit for bit with the oracle
stepping that system by itself (the stated 1e-9 relative tolerance is asserted too),
together with its level-0 encounter list and the summed SyMBA statistics.  The mixed
path is checked for energy and angular-momentum conservation against the FP64 path.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import _lib as L
from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300.api import Ensemble

pytestmark = pytest.mark.gpu


def _compact(name, nsys, scale, tp_per_pl):
    # compact disks (0.8-1.2 AU, heavier bodies) so that SyMBA systems meet encounters
    return IC.make_ensemble(name, nsys=nsys, scale=scale, tp_per_pl=tp_per_pl, amin=0.8, amax=1.2, mmin=1e-9,
                            mmax=1e-6)


def _oracles(E, **kw):
    cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
    return [O.OracleSystem(E["integrator"], cb, pl, tp if len(tp["rh"]) else None, **kw) for pl, tp in E["systems"]]


def _check_states(ens, refs, tol=1e-9):
    rh, vh, st = ens.get_pl()
    trh, tvh, tst = ens.get_tp()
    exact = True
    for s, ref in enumerate(refs):
        a, b = ens.poff[s], ens.poff[s + 1]
        r_rh, r_vh, r_st = ref.get_pl()
        assert np.array_equal(st[a:b], r_st)
        pairs = [(rh[a:b], r_rh), (vh[a:b], r_vh)]
        if ens.ntp[s]:
            a, b = ens.toff[s], ens.toff[s + 1]
            o_rh, o_vh, o_st = ref.get_tp()
            assert np.array_equal(tst[a:b], o_st)
            pairs += [(trh[a:b], o_rh), (tvh[a:b], o_vh)]
        for x, y in pairs:
            rel = np.linalg.norm(x - y, axis=1) / np.linalg.norm(y, axis=1)
            assert rel.max() <= tol, (s, rel.max())
            exact = exact and np.array_equal(x, y)
    return exact


def test_symba_ensemble_fp64_bitexact(ctx):
    E = _compact("C4", nsys=7, scale=0.04, tp_per_pl=2)
    kw = dict(dt=0.005, rhscale=3.0)
    ens = Ensemble(ctx, E, precision="FP64", **kw)
    refs = _oracles(E, **kw)
    for _ in range(4):
        ens.step(25)
        for ref in refs:
            ref.step(25)
        for s, ref in enumerate(refs):
            gi = ens.plpl_list(s)
            ri = ref.plpl_list()
            assert all(np.array_equal(a, b) for a, b in zip(gi, ri)), s
    assert _check_states(ens, refs)
    st = ens.stats()
    rs = [r.stats() for r in refs]
    assert st["system_steps_with_encounters"] == sum(r["steps_with_encounters"] for r in rs)
    assert st["plpl_encounters"] == sum(r["plpl_encounters"] for r in rs)
    assert st["pltp_encounters"] == sum(r["pltp_encounters"] for r in rs)
    assert st["max_recursion"] == max(r["max_recursion"] for r in rs)
    assert st["recursion_substeps"] == sum(r["recursion_substeps"] for r in rs)
    assert st["system_steps_with_encounters"] > 0 and st["max_recursion"] >= 1
    eg = ens.energy()
    for s, ref in enumerate(refs):
        er = ref.energy()
        assert abs(eg["te"][s] - er["te"]) <= 1e-12 * abs(er["te"])


def test_helio_ensemble_fp64_bitexact(ctx):
    E = IC.make_ensemble("C3", nsys=9, scale=0.08)
    kw = dict(dt=0.01)
    ens = Ensemble(ctx, E, precision="FP64", **kw)
    refs = _oracles(E, rhscale=6.5, **kw)
    ens.step(150)
    for ref in refs:
        ref.step(150)
    assert _check_states(ens, refs)


def test_whm_ensemble_fp64_bitexact(ctx):
    # batched WHM (Jacobi coordinates per system, serial sums in the reference's order)
    E = IC.make_ensemble("C3", nsys=9, scale=0.08, integrator="WHM")
    kw = dict(dt=0.01)
    ens = Ensemble(ctx, E, precision="FP64", **kw)
    refs = _oracles(E, **kw)
    ens.step(150)
    for ref in refs:
        ref.step(150)
    assert _check_states(ens, refs)
    eg = ens.energy()
    for s, ref in enumerate(refs):
        er = ref.energy()
        assert abs(eg["te"][s] - er["te"]) <= 1e-12 * abs(er["te"])


def test_whm_ensemble_mixed(ctx):
    # mixed WHM: graph replay gives the eager bits; energy error within 2x of the FP64 path's
    E = IC.make_ensemble("C3", nsys=6, scale=0.1, integrator="WHM")
    out, dE = [], {}
    for prec, graphs in (("MIXED", True), ("MIXED", False), ("FP64", True)):
        ens = Ensemble(ctx, E, precision=prec, dt=0.01)
        ens.use_graphs(graphs)
        e0 = ens.energy()
        ens.step(300)
        e1 = ens.energy()
        dE[(prec, graphs)] = np.abs((e1["te"] - e0["te"]) / e0["te"])
        out.append(ens.get_pl() + ens.get_tp())
        ens.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    assert np.all(dE[("MIXED", True)] < np.maximum(2 * dE[("FP64", True)], 1e-10)), (dE[("MIXED", True)],
                                                                                    dE[("FP64", True)])


def test_symba_ensemble_uneven_sizes(ctx):
    # systems of very different sizes (2 .. 300 bodies, tp-free and tp-carrying) in one ensemble
    parts = [IC.make_system(seed=s, npl=n, ntp=t, amin=0.8, amax=1.2, mmin=1e-9, mmax=1e-6)
             for s, (n, t) in enumerate([(2, 0), (300, 0), (17, 40), (129, 1), (64, 0)])]
    systems = [(IC.sort_for_integrator(pl, "SYMBA"), tp) for _, pl, tp in parts]
    E = {"integrator": "SYMBA", "dt": 0.005, "rhscale": 3.0,
         "npl": np.array([len(p["Gmass"]) for p, _ in systems], np.int32),
         "ntp": np.array([len(t["rh"]) for _, t in systems], np.int32),
         "GMcb": np.full(len(systems), IC.GMCB), "Rcb": np.full(len(systems), IC.RCB),
         "pl": {k: np.concatenate([p[k] for p, _ in systems]) for k in ("rh", "vh", "Gmass", "radius", "rhill")},
         "tp": {k: np.concatenate([t[k] for _, t in systems]) for k in ("rh", "vh")}, "systems": systems}
    ens = Ensemble(ctx, E, precision="FP64")
    refs = _oracles(E, dt=0.005, rhscale=3.0)
    ens.step(60)
    for ref in refs:
        ref.step(60)
    assert _check_states(ens, refs)


def test_symba_ensemble_mixed_conservation(ctx):
    E = _compact("C4", nsys=5, scale=0.06, tp_per_pl=0)
    kw = dict(dt=0.005, rhscale=2.0)
    f = Ensemble(ctx, E, precision="FP64", **kw)
    m = Ensemble(ctx, E, precision="MIXED", **kw)
    e0 = f.energy()
    f.step(300)
    m.step(300)
    ef, em = f.energy(), m.energy()
    dEf = np.abs(ef["te_helio"] - e0["te_helio"]) / np.abs(e0["te_helio"])
    dEm = np.abs(em["te_helio"] - e0["te_helio"]) / np.abs(e0["te_helio"])
    dLm = np.linalg.norm(em["L"] - e0["L"], axis=1) / np.linalg.norm(e0["L"], axis=1)
    assert np.all(dEm < np.maximum(2 * dEf, 1e-9)), (dEm, dEf)
    assert np.all(dLm < 1e-9)
    assert f.stats()["plpl_encounters"] > 0


@pytest.mark.parametrize("tile,group,scale", [(64, 1, 0.06), (128, 1, 0.06), (128, 2, 0.06), (128, 4, 0.06),
                                              (128, 2, 0.2), (128, 4, 0.2)])
def test_symba_ensemble_mixed_conservation_tiles(ctx, tile, group, scale):
    # both tile sizes and the row groups of the symmetric pl-pl kick through whole SyMBA
    # steps (the closing kick split by the items' encounter flags; groups wider than a
    # system's tiles, and systems of several groups): energy within 2x of the FP64 path's error
    E = _compact("C4", nsys=5, scale=scale, tp_per_pl=0)
    kw = dict(dt=0.005, rhscale=2.0)
    f = Ensemble(ctx, E, precision="FP64", **kw)
    m = Ensemble(ctx, E, precision="MIXED", **kw)
    m.set_kick_tile(tile)
    m.set_kick_group(group)
    e0 = f.energy()
    nstep = 100 if scale < 0.1 else 40
    f.step(nstep)
    m.step(nstep)
    assert m.kick_tile() == tile and m.kick_group() == group
    ef, em = f.energy(), m.energy()
    dEf = np.abs(ef["te_helio"] - e0["te_helio"]) / np.abs(e0["te_helio"])
    dEm = np.abs(em["te_helio"] - e0["te_helio"]) / np.abs(e0["te_helio"])
    assert np.all(dEm < np.maximum(2 * dEf, 1e-9)), (dEm, dEf)
    assert f.stats()["plpl_encounters"] > 0


def test_symba_ensemble_lists_many_tiles(ctx):
    # systems of 150-1500 bodies (many 64-body tiles, radius-sorted culling active), lists
    # checked against the oracle's all-pairs check at every step across a re-sort boundary
    E = IC.make_ensemble("C4", nsys=4, scale=0.3)
    kw = dict(dt=0.002, rhscale=4.0)
    ens = Ensemble(ctx, E, precision="FP64", **kw)
    refs = _oracles(E, **kw)
    total = 0
    for _ in range(12):
        ens.step(1)
        for s, ref in enumerate(refs):
            ref.step(1)
            gi = ens.plpl_list(s)
            ri = ref.plpl_list()
            assert all(np.array_equal(a, b) for a, b in zip(gi, ri)), s
            total += len(ri[0])
    assert total > 0
    assert _check_states(ens, refs)


def test_helio_ensemble_graph_replay_matches_eager(ctx):
    # HELIO steps replayed from a captured CUDA graph give the same bits as eager steps
    E = IC.make_ensemble("C3", nsys=6, scale=0.1)
    out = []
    for graphs in (True, False):
        ens = Ensemble(ctx, E, precision="MIXED", dt=0.01)
        ens.use_graphs(graphs)
        ens.step(40)
        out.append(ens.get_pl() + ens.get_tp())
        ens.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_mixed_kick_shapes_identical(ctx):
    # every broadcast tile shape of the batched mixed kick gives the same bits (pl-pl with
    # the radius guard and pl-tp, systems of uneven sizes spanning several tiles); the
    # default runs the symmetric pl-pl kernel and an autotuned pl-tp shape
    E = IC.make_ensemble("C4", nsys=5, scale=0.15, tp_per_pl=1)
    out = []
    for v in list(range(5)) + [-1]:
        ens = Ensemble(ctx, E, precision="MIXED", dt=0.005, rhscale=3.0)
        ens.set_kick_variant(v)
        assert ens.kick_variant() == {"pl": -1, "tp": -1}
        ens.step(20)
        kv = ens.kick_variant()
        if v >= 0:
            assert kv == {"pl": v, "tp": v}
        else:
            assert kv["pl"] == L.SWG_KICK_SYMMETRIC and 0 <= kv["tp"] < 5
        out.append(ens.get_pl() + ens.get_tp())
        ens.close()
    for other in out[1:5]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b)
    for a, b in zip(out[0][:2], out[5][:2]):  # pl rh, vh: the same sums in another order
        rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(a, axis=1)
        assert rel.max() < 1e-9, rel.max()


def _pack(E, systems):
    # the ensemble dict of E with its systems replaced
    E = dict(E)
    E["systems"] = systems
    E["npl"] = np.array([len(pl["Gmass"]) for pl, _ in systems], np.int32)
    E["ntp"] = np.array([len(tp["rh"]) for _, tp in systems], np.int32)
    E["pl"] = {k: np.concatenate([pl[k] for pl, _ in systems]) for k in ("rh", "vh", "Gmass", "radius", "rhill")}
    E["tp"] = {k: np.concatenate([tp[k] for _, tp in systems]) for k in ("rh", "vh")}
    return E


@pytest.mark.parametrize("integrator,lclose", [("SYMBA", True), ("HELIO", False)])
def test_ensemble_getacch_mixed_tolerance(ctx, integrator, lclose):
    # pair accelerations of every system (symmetric and broadcast kernels) against the oracle's
    # FP64 triangular kick; systems of 2 to ~700 bodies, tiles partly filled, an overlapping pair
    E = IC.make_ensemble("C4", nsys=6, scale=0.3)
    E["integrator"] = integrator
    sysl = [({k: v.copy() for k, v in pl.items()}, tp) for pl, tp in E["systems"]]
    pl1 = sysl[1][0]  # 279 bodies: pairs within the radii inside a tile and across tiles
    for i, j in [(3, 7), (20, 270), (150, 100)]:
        pl1["rh"][j] = pl1["rh"][i] + 1e-6 * np.array([0.6, -0.48, 0.64])
        pl1["radius"][[i, j]] = 1e-5
    sysl[2] = ({k: v[:2].copy() for k, v in sysl[2][0].items()}, sysl[2][1])
    E = _pack(E, sysl)
    rad = integrator == "SYMBA" or lclose
    want = [O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"] if rad else None) for pl, _ in sysl]
    for v in (-1, 1):
        ens = Ensemble(ctx, E, precision="MIXED", dt=0.005, lclose=lclose)
        ens.set_kick_variant(v)
        g = ens.getacch_int_pl()
        for s, r in enumerate(want):
            a, b = ens.poff[s], ens.poff[s + 1]
            e = np.linalg.norm(g[a:b] - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-300)
            # FP32 pair terms with float-float partial sums: 2e-5 max, 1e-6 RMS per body
            assert e.max() < 2e-5, (v, s, e.max())
            assert np.sqrt(np.mean(e ** 2)) < 1e-6, (v, s)
        g2 = ens.getacch_int_pl()
        assert np.array_equal(g, g2)  # deterministic
        ens.close()


@pytest.mark.parametrize("strip", [1, 2, 4, 8, 16, 0])
def test_symmetric_kick_strips(ctx, strip):
    # every strip length of the symmetric pl-pl kick (forced, and the autotuned default):
    # within the mixed-kick tolerance of the oracle's FP64 triangular kick, and deterministic
    E = IC.make_ensemble("C4", nsys=4, scale=0.5)
    want = [O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"]) for pl, _ in E["systems"]]
    ens = Ensemble(ctx, E, precision="MIXED")
    ens.set_kick_strip(strip)
    g = ens.getacch_int_pl()
    used = ens.kick_strip()
    assert used == strip if strip else used in (1, 2, 4, 8, 16)
    for s, r in enumerate(want):
        a, b = ens.poff[s], ens.poff[s + 1]
        e = np.linalg.norm(g[a:b] - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-300)
        assert e.max() < 2e-5, (strip, s, e.max())
        assert np.sqrt(np.mean(e ** 2)) < 1e-6, (strip, s)
    assert np.array_equal(g, ens.getacch_int_pl())
    ens.close()


@pytest.mark.parametrize("tile,strip", [(64, 1), (64, 4), (64, 16), (0, 0)])
def test_symmetric_kick_tiles(ctx, tile, strip):
    # 64-body tiles of the symmetric pl-pl kick (and the autotuned default): within the
    # mixed-kick tolerance of the oracle's FP64 triangular kick, and deterministic
    E = IC.make_ensemble("C4", nsys=4, scale=0.5)
    want = [O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"]) for pl, _ in E["systems"]]
    ens = Ensemble(ctx, E, precision="MIXED")
    ens.set_kick_tile(tile)
    ens.set_kick_strip(strip)
    g = ens.getacch_int_pl()
    assert ens.kick_tile() == tile if tile else ens.kick_tile() in (64, 128)
    for s, r in enumerate(want):
        a, b = ens.poff[s], ens.poff[s + 1]
        e = np.linalg.norm(g[a:b] - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-300)
        assert e.max() < 2e-5, (tile, strip, s, e.max())
        assert np.sqrt(np.mean(e ** 2)) < 1e-6, (tile, strip, s)
    assert np.array_equal(g, ens.getacch_int_pl())
    ens.close()


@pytest.mark.parametrize("group,strip", [(2, 2), (2, 4), (2, 8), (4, 1), (4, 4), (4, 8), (4, 16), (1, 4)])
def test_symmetric_kick_groups(ctx, group, strip):
    # row groups of the symmetric pl-pl kick (a block of `group` warps per item, one pair slot
    # per group and tile J): within the mixed-kick tolerance of the oracle's FP64 triangular
    # kick, deterministic, and reported as the plan in use
    E = IC.make_ensemble("C4", nsys=4, scale=0.5)
    want = [O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"]) for pl, _ in E["systems"]]
    ens = Ensemble(ctx, E, precision="MIXED")
    ens.set_kick_group(group)
    ens.set_kick_strip(strip)
    g = ens.getacch_int_pl()
    assert ens.kick_group() == group and ens.kick_strip() == strip
    assert group == 1 or (ens.kick_tile() == 128 and ens.kick_warps() == group)
    for s, r in enumerate(want):
        a, b = ens.poff[s], ens.poff[s + 1]
        e = np.linalg.norm(g[a:b] - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-300)
        assert e.max() < 2e-5, (group, strip, s, e.max())
        assert np.sqrt(np.mean(e ** 2)) < 1e-6, (group, strip, s)
    assert np.array_equal(g, ens.getacch_int_pl())
    ens.close()


@pytest.mark.parametrize("warps", [2, 4, 0])
def test_symmetric_kick_warps_same_bits(ctx, warps):
    # warps per block of the symmetric pl-pl kick (forced, and the autotuned default): every
    # warp is an independent worker of the persistent grid, so each count gives the bits of
    # one warp per block at the same tile and strip
    E = IC.make_ensemble("C4", nsys=4, scale=0.5)

    def accel(w):
        ens = Ensemble(ctx, E, precision="MIXED")
        ens.set_kick_tile(128)
        ens.set_kick_strip(4)
        ens.set_kick_warps(w)
        g = ens.getacch_int_pl()
        used = ens.kick_warps()
        ens.close()
        return g, used

    g1, used1 = accel(1)
    g, used = accel(warps)
    assert used1 == 1 and (used == warps if warps else used in (1, 2, 4))
    assert np.array_equal(g, g1)


def test_mixed_drift_matches_fp64_drift(ctx):
    # massless bodies feel no pair forces and move the central body not at all, so the
    # mixed and FP64 ensembles differ only in the drift: the fast FP64 solver form of the
    # mixed path against the reference form, over circular, eccentric and hyperbolic orbits
    E = IC.make_ensemble("C3", nsys=4, scale=0.1)
    sysl = []
    for s, (pl, tp) in enumerate(E["systems"]):
        pl = {k: v.copy() for k, v in pl.items()}
        pl["Gmass"][:] = 0.0
        pl["rhill"][:] = 0.0
        f = np.linspace(0.3, 1.5, len(pl["Gmass"]))  # speed factors: e up to ~0.9, hyperbolic above sqrt(2)
        pl["vh"] = pl["vh"] * f[:, None]
        sysl.append((pl, tp))
    E = _pack(E, sysl)
    out = []
    for prec in ("FP64", "MIXED"):
        ens = Ensemble(ctx, E, precision=prec, dt=0.01, lclose=False)
        ens.step(100)
        out.append(ens.get_pl() + ens.get_tp())
        ens.close()
    for a, b in zip(out[0][:2] + out[0][3:5], out[1][:2] + out[1][3:5]):
        rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(a, axis=1)
        assert rel.max() < 1e-12, rel.max()


@pytest.mark.parametrize("integrator", ["HELIO", "WHM"])
def test_ensemble_ragged_and_empty_systems(ctx, integrator):
    # systems with no massive body (test particles around the central body only), one massive
    # body, no test particles, and ordinary ones, in one ensemble; FP64 against the oracle,
    # mixed runs to completion with finite states
    sizes = [(0, 5), (1, 0), (3, 2), (40, 0), (25, 30)]
    systems = []
    for s, (n, t) in enumerate(sizes):
        _, pl, tp = IC.make_system(seed=20 + s, npl=max(n, 1), ntp=t)
        pl = {k: v[:n].copy() for k, v in IC.sort_for_integrator(pl, integrator).items()}
        systems.append((pl, tp))
    E = _pack({"integrator": integrator, "dt": 0.01, "rhscale": 6.5, "GMcb": np.full(len(sizes), IC.GMCB),
               "Rcb": np.full(len(sizes), IC.RCB)}, systems)
    ens = Ensemble(ctx, E, precision="FP64", dt=0.01)
    refs = [O.OracleSystem(integrator, {"Gmass": IC.GMCB, "radius": IC.RCB}, pl, tp if len(tp["rh"]) else None,
                           dt=0.01) for pl, tp in systems]
    ens.step(50)
    for r in refs:
        r.step(50)
    rh, vh, st = ens.get_pl()
    trh, tvh, tst = ens.get_tp()
    for s, r in enumerate(refs):
        a, b = ens.poff[s], ens.poff[s + 1]
        if b > a:
            o_rh, o_vh, _ = r.get_pl()
            assert np.array_equal(rh[a:b], o_rh) and np.array_equal(vh[a:b], o_vh), s
        a, b = ens.toff[s], ens.toff[s + 1]
        if b > a:
            o_rh, o_vh, _ = r.get_tp()
            assert np.array_equal(trh[a:b], o_rh) and np.array_equal(tvh[a:b], o_vh), s
    ens.close()
    m = Ensemble(ctx, E, precision="MIXED", dt=0.01)
    m.step(50)
    out = m.get_pl() + m.get_tp()
    assert all(np.all(np.isfinite(x)) for x in out)
    m.close()


@pytest.mark.parametrize("integrator", ["SYMBA", "SYMBA_COLL", "HELIO", "WHM"])
def test_stream_schedules_match_serial(ctx, integrator):
    # The overlapped step (side streams: SyMBA level-0 drift and closing-kick items beside
    # the recursion, HELIO test-particle groups, WHM test-particle drift) gives the same bits
    # as the serial step that the per-class profile runs; SYMBA_COLL inflates the radii so
    # that the recursion pauses for perfect merges on the host.
    if integrator.startswith("SYMBA"):
        E = _compact("C4", nsys=6, scale=0.25, tp_per_pl=1)
        if integrator == "SYMBA_COLL":
            E["pl"]["radius"] = E["pl"]["radius"] * 300.0
            E["systems"] = None
        kw = dict(dt=0.005, rhscale=3.0)
    else:
        E = IC.make_ensemble("C3", nsys=8, scale=0.2, integrator=integrator)
        kw = dict(dt=0.01)
    out, stats = [], None
    for prof in (False, True):
        ens = Ensemble(ctx, E, precision="MIXED", **kw)
        ens.profile(prof)
        ens.step(25)
        out.append(ens.get_pl() + ens.get_tp())
        stats = ens.stats()
        ens.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    if integrator.startswith("SYMBA"):
        assert stats["plpl_encounters"] > 0
    if integrator == "SYMBA_COLL":
        assert stats["collisions"] > 0


def _gmtiny_ensemble():
    # compact disks with a GMTINY threshold at each system's median G*m: the lighter half of
    # every system (which the Gmass-descending order puts last) is semi-interacting
    E = _compact("C4", nsys=4, scale=0.05, tp_per_pl=1)
    gmtiny = float(np.median(E["pl"]["Gmass"]))
    return E, gmtiny


def test_symba_gmtiny_fp64_bitexact(ctx):
    # GMTINY (symba_util.f90:175-208 and the nplm loop bounds): single systems and one ensemble,
    # each system against the oracle stepping it alone (FP64, bit for bit, level-0 lists too)
    from swiftest_gb300.api import NBodySystem
    E, gmtiny = _gmtiny_ensemble()
    kw = dict(dt=0.005, rhscale=3.0)
    cb = {"Gmass": IC.GMCB, "radius": IC.RCB}
    refs = [O.OracleSystem("SYMBA", cb, pl, tp, gmtiny=gmtiny, **kw) for pl, tp in E["systems"]]
    ens = Ensemble(ctx, E, precision="FP64", gmtiny=gmtiny, **kw)
    singles = [NBodySystem(ctx, "SYMBA", cb, pl, tp, gmtiny=gmtiny, precision="FP64", **kw) for pl, tp in E["systems"]]
    for _ in range(4):
        ens.step(25)
        for s, ref in enumerate(refs):
            ref.step(25)
            singles[s].step(25)
            ri = ref.plpl_list()
            assert all(np.array_equal(a, b) for a, b in zip(ens.plpl_list(s), ri)), s
            assert all(np.array_equal(a, b) for a, b in zip(singles[s].plpl_list(), ri)), s
    assert _check_states(ens, refs)
    for s, ref in enumerate(refs):
        assert np.array_equal(singles[s].get_pl()[0], ref.get_pl()[0]), s
        assert np.array_equal(singles[s].get_tp()[0], ref.get_tp()[0]), s
        singles[s].close()
    assert ens.stats()["plpl_encounters"] > 0


def test_symba_gmtiny_mixed(ctx):
    # the mixed path with GMTINY: the broadcast pl-pl kernel with the semi-interacting rule
    # (within the mixed-kick tolerance of the oracle's nplm kick) and the energy error within
    # 2x of the FP64 path's
    E, gmtiny = _gmtiny_ensemble()
    kw = dict(dt=0.005, rhscale=3.0)
    m = Ensemble(ctx, E, precision="MIXED", gmtiny=gmtiny, **kw)
    g = m.getacch_int_pl()
    assert m.kick_variant()["pl"] != L.SWG_KICK_SYMMETRIC
    for s, (pl, _) in enumerate(E["systems"]):
        nplm = int(np.sum(pl["Gmass"] >= gmtiny))
        assert nplm < len(pl["Gmass"])
        r = O.kick_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], nplm=nplm)
        a, b = m.poff[s], m.poff[s + 1]
        e = np.linalg.norm(g[a:b] - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-300)
        assert e.max() < 2e-5, (s, e.max())
    f = Ensemble(ctx, E, precision="FP64", gmtiny=gmtiny, **kw)
    e0 = f.energy()
    f.step(200)
    m.step(200)
    ef, em = f.energy(), m.energy()
    dEf = np.abs(ef["te_helio"] - e0["te_helio"]) / np.abs(e0["te_helio"])
    dEm = np.abs(em["te_helio"] - e0["te_helio"]) / np.abs(e0["te_helio"])
    assert np.all(dEm < np.maximum(2 * dEf, 1e-9)), (dEm, dEf)


def test_gmtiny_ensemble_rejects_sortsweep(ctx):
    E, gmtiny = _gmtiny_ensemble()
    with pytest.raises(L.SwiftestGB300Error):
        Ensemble(ctx, E, precision="FP64", gmtiny=gmtiny, encounter_check_plpl="SORTSWEEP")
