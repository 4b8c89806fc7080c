"""NetCDF output frames and restart (swiftest_gb300.netcdf) against the reference's data.nc layout.

CPU tests write frames from host arrays and read them back: the dimension and variable
names of swiftest_io_netcdf_initialize_output (src/swiftest/swiftest_io.f90:821-1000), the
slot order (central body, massive bodies, test particles), the particle types, mass = Gmass /
GU, the energy variables, and the restart selection of swiftest_io_netcdf_get_valid_masks
(:1190-1279: status not INACTIVE; Gmass > 0 massive, else test particle).  The GPU test writes
frames of a stepped system (with orbital elements from the GPU) and restarts from the last.
"""
import numpy as np
import pytest

pytest.importorskip("scipy")
from swiftest_gb300 import netcdf as N  # noqa: E402


def _frame(rng, npl, ntp):
    return {"rh": rng.normal(size=(npl, 3)), "vh": rng.normal(size=(npl, 3)), "status": np.zeros(npl, np.int32),
            "Gmass": 10 ** rng.uniform(-10, -6, npl), "radius": rng.uniform(1e-6, 1e-5, npl),
            "rhill": rng.uniform(1e-4, 1e-3, npl), "trh": rng.normal(size=(ntp, 3)), "tvh": rng.normal(size=(ntp, 3)),
            "tstatus": np.zeros(ntp, np.int32)}


def test_frames_round_trip_and_layout(tmp_path):
    from scipy.io import netcdf_file
    rng = np.random.default_rng(1)
    cb = {"name": "Sun", "Gmass": N.GU_AU_MSUN_YR, "radius": 0.00465, "j2rp2": 1e-7, "j4rp4": 0.0}
    npl, ntp = 5, 7
    frames = [_frame(rng, npl, ntp) for _ in range(3)]
    frames[2]["status"][1] = N.INACTIVE  # a merged body keeps its slot
    frames[2]["tstatus"][3] = N.INACTIVE
    energy = {"ke": 1.0, "pe": -3.0, "be": 0.0, "te": -2.0, "L": np.array([0.1, 0.2, 0.3]), "E_collisions": 1e-9,
              "L_escape": np.zeros(3)}
    p = tmp_path / "data.nc"
    with N.NetCDFOutput(p, cb, npl, ntp, out_form="XV", gmtiny=1e-8) as out:
        for k, fr in enumerate(frames):
            out.write_arrays(0.5 * k, dict(fr, energy=energy))
    with netcdf_file(str(p), "r", mmap=False) as f:
        assert set(f.dimensions) == {"time", "space", "name", "string32"}
        assert f.dimensions["time"] is None and f.dimensions["name"] == 1 + npl + ntp
        for v in ("time", "space", "name", "id", "particle_type", "status", "npl", "ntp", "nplm", "rh", "vh", "Gmass",
                  "mass", "rhill", "radius", "j2rp2", "j4rp4", "KE_orb", "PE", "TE", "L_orbit", "L_escape",
                  "E_collisions"):
            assert v in f.variables, v
        assert f.variables["rh"].dimensions == ("time", "name", "space")
        assert list(f.variables["id"][:]) == list(range(1 + npl + ntp))
        assert np.array_equal(f.variables["npl"][:], [npl, npl, npl - 1])
        assert np.array_equal(f.variables["ntp"][:], [ntp, ntp, ntp - 1])
        types = N._strings(f.variables["particle_type"][:])
        tiny = frames[0]["Gmass"] <= 1e-8
        assert types[0] == N.CB_TYPE and types[1 + npl:] == [N.TP_TYPE] * ntp
        assert types[1:1 + npl] == [N.PL_TINY_TYPE if t else N.PL_TYPE for t in tiny]
        assert np.allclose(f.variables["mass"][1][1:1 + npl], frames[1]["Gmass"] / N.GU_AU_MSUN_YR, rtol=1e-15)
        assert f.variables["TE"][2] == -2.0 and np.array_equal(f.variables["L_orbit"][0], [0.1, 0.2, 0.3])
    got = N.read_frame(p)  # the last frame: the inactive bodies are left out
    fr = frames[2]
    keep, tkeep = fr["status"] != N.INACTIVE, fr["tstatus"] != N.INACTIVE
    assert got["time"] == 1.0 and got["tslot"] == 2
    assert np.array_equal(got["pl"]["rh"], fr["rh"][keep]) and np.array_equal(got["pl"]["vh"], fr["vh"][keep])
    assert np.array_equal(got["pl"]["Gmass"], fr["Gmass"][keep])
    assert np.array_equal(got["pl"]["radius"], fr["radius"][keep])
    assert np.array_equal(got["tp"]["rh"], fr["trh"][tkeep]) and np.array_equal(got["tp"]["vh"], fr["tvh"][tkeep])
    assert list(got["pl"]["id"]) == [1 + i for i in np.flatnonzero(keep)]
    assert got["cb"]["Gmass"] == cb["Gmass"] and got["cb"]["name"] == "Sun"
    first = N.read_frame(p, 0)
    assert np.array_equal(first["pl"]["rh"], frames[0]["rh"]) and len(first["tp"]["rh"]) == ntp


def test_elements_need_a_context(tmp_path):
    rng = np.random.default_rng(2)
    cb = {"Gmass": N.GU_AU_MSUN_YR, "radius": 0.00465}
    with N.NetCDFOutput(tmp_path / "el.nc", cb, 2, 0, out_form="EL") as out:
        with pytest.raises(ValueError):
            out.write_arrays(0.0, _frame(rng, 2, 0))
    with pytest.raises(ValueError):
        N.NetCDFOutput(tmp_path / "bad.nc", cb, 2, 0, out_form="XYZ")


@pytest.mark.gpu
def test_system_frames_and_restart(ctx, tmp_path):
    from swiftest_gb300 import initial_conditions as IC
    from swiftest_gb300.api import NBodySystem
    cb, pl, tp = IC.make_system(seed=5, npl=40, ntp=60, amin=0.8, amax=1.2, mmin=1e-9, mmax=1e-6)
    pl = IC.sort_for_integrator(pl, "SYMBA")
    kw = dict(dt=0.005, rhscale=3.0, lclose=True)
    s = NBodySystem(ctx, "SYMBA", cb, pl, tp, **kw)
    cbd = {"name": "Sun", "Gmass": cb["Gmass"], "radius": cb["radius"]}
    p = tmp_path / "data.nc"
    with N.NetCDFOutput(p, cbd, s.npl, s.ntp, out_form="XVEL") as out:
        out.write_frame(0.0, s)
        for k in range(1, 4):
            s.step(10)
            out.write_frame(0.05 * k, s)
    fr = N.read_frame(p)
    rh, vh, st = s.get_pl()
    keep = st != N.INACTIVE
    assert np.array_equal(fr["pl"]["rh"], rh[keep]) and np.array_equal(fr["pl"]["vh"], vh[keep])
    trh, tvh, tst = s.get_tp()
    assert np.array_equal(fr["tp"]["rh"], trh[tst != N.INACTIVE])
    # orbital elements of the frame: the GPU's xv2el, angles in degrees
    from scipy.io import netcdf_file
    with netcdf_file(str(p), "r", mmap=False) as f:
        a, inc = np.array(f.variables["a"][3]), np.array(f.variables["inc"][3])
    el = ctx.xv2el(cb["Gmass"] + fr["pl"]["Gmass"], fr["pl"]["rh"], fr["pl"]["vh"])
    assert np.array_equal(a[1:1 + s.npl][keep], el["a"]) and np.allclose(inc[1:1 + s.npl][keep], el["inc"] * N.RAD2DEG)
    # restart from the last frame: the same state, and the next steps stay with the running system
    r = NBodySystem(ctx, "SYMBA", fr["cb"], fr["pl"], fr["tp"], **kw)
    s.step(20)
    r.step(20)
    a1, b1 = s.get_pl()[0][keep], r.get_pl()[0]
    rel = np.linalg.norm(a1 - b1, axis=1) / np.linalg.norm(a1, axis=1)
    assert rel.max() < 1e-10, rel.max()


def test_load_run_from_a_netcdf_frame(tmp_path):
    # IN_TYPE NETCDF_DOUBLE: the run starts from the last frame of NC_IN
    from swiftest_gb300 import io
    rng = np.random.default_rng(3)
    cb = {"name": "Sun", "Gmass": N.GU_AU_MSUN_YR, "radius": 0.00465}
    fr = _frame(rng, 4, 3)
    with N.NetCDFOutput(tmp_path / "init_cond.nc", cb, 4, 3, out_form="XV", lenergy=False) as out:
        out.write_arrays(2.5, fr)
    (tmp_path / "param.in").write_text("IN_TYPE NETCDF_DOUBLE\nNC_IN init_cond.nc\n")
    run = io.load_run(tmp_path / "param.in")
    assert run["time"] == 2.5 and run["cb"]["Gmass"] == cb["Gmass"]
    assert np.array_equal(run["pl"]["rh"], fr["rh"]) and np.array_equal(run["tp"]["vh"], fr["tvh"])
