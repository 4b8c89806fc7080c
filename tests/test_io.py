"""ASCII initial-condition files (IN_TYPE ASCII, the reference's swiftest_io readers):
write/read round trips, the parameter reader, element files converted on the GPU."""
import numpy as np
import pytest

from swiftest_gb300 import initial_conditions as IC
from swiftest_gb300 import io


def _run_dir(tmp_path, form="XV"):
    cb, pl, tp = IC.make_system(seed=3, npl=12, ntp=5)
    pl = IC.sort_for_integrator(pl, "HELIO")
    (tmp_path / "param.in").write_text(
        "! comment line\n" + "t0 0.0\nDT 0.01\nIN_TYPE ASCII\n" + f"IN_FORM {form}\n" +
        "CB_IN cb.in\nPL_IN pl.in\nTP_IN tp.in\nCHK_CLOSE YES\nRHILL_PRESENT yes\nROTATION NO\n")
    io.write_cb(tmp_path / "cb.in", {"name": "Sun", "Gmass": IC.GMCB, "radius": IC.RCB})
    return cb, pl, tp


def test_ascii_xv_round_trip(tmp_path):
    cb, pl, tp = _run_dir(tmp_path)
    io.write_bodies(tmp_path / "pl.in", pl, "pl", rhill_present=True, lclose=True)
    io.write_bodies(tmp_path / "tp.in", tp, "tp")
    run = io.load_run(tmp_path / "param.in")
    assert run["param"]["DT"] == "0.01" and io.flag(run["param"], "chk_close") and not io.flag(run["param"], "GR")
    assert run["cb"]["Gmass"] == IC.GMCB and run["cb"]["radius"] == IC.RCB and run["cb"]["name"] == "Sun"
    for k in ("Gmass", "rhill", "radius", "rh", "vh"):
        assert np.array_equal(run["pl"][k], pl[k]), k
    for k in ("rh", "vh"):
        assert np.array_equal(run["tp"][k], tp[k]), k
    assert len(run["pl"]["name"]) == 12 and len(run["tp"]["name"]) == 5


def test_ascii_el_parsing_degrees(tmp_path):
    (tmp_path / "pl.in").write_text("!! header\n2\nA 1e-6 0.01\n1e-5\n1.0 0.1 10.0\n20.0 30.0 40.0\n"
                                    "B 2e-6 0.02\n2e-5\n2.0 0.2 0.0\n0.0 90.0 180.0\n")
    b = io.read_bodies(tmp_path / "pl.in", "pl", "EL", rhill_present=True, lclose=True)
    np.testing.assert_array_equal(b["a"], [1.0, 2.0])
    np.testing.assert_allclose(b["inc"], np.radians([10.0, 0.0]))
    np.testing.assert_allclose(b["capm"], np.radians([40.0, 180.0]))
    assert b["radius"][1] == 2e-5 and b["rhill"][0] == 0.01
    with pytest.raises(ValueError):
        io.read_bodies(tmp_path / "pl.in", "pl", "XX")


@pytest.mark.gpu
def test_ascii_el_run_converted_on_gpu(ctx, tmp_path):
    from oracle import oracle as O
    _run_dir(tmp_path, form="EL")
    (tmp_path / "pl.in").write_text("2\nA 1e-6 0.01\n1e-5\n1.0 0.1 10.0\n20.0 30.0 40.0\n"
                                    "B 2e-6 0.02\n2e-5\n2.0 0.2 5.0\n0.0 90.0 180.0\n")
    (tmp_path / "tp.in").write_text("1\nT1\n3.0 0.05 2.0\n10.0 20.0 30.0\n")
    run = io.load_run(tmp_path / "param.in", ctx=ctx)
    pl = run["pl"]
    r_rh, r_vh = O.el2xv(IC.GMCB + pl["Gmass"], pl["a"], pl["e"], pl["inc"], pl["capom"], pl["omega"], pl["capm"])
    np.testing.assert_allclose(pl["rh"], r_rh, rtol=1e-12)
    np.testing.assert_allclose(pl["vh"], r_vh, rtol=1e-12)
    tp = run["tp"]
    t_rh, _ = O.el2xv(IC.GMCB, tp["a"], tp["e"], tp["inc"], tp["capom"], tp["omega"], tp["capm"])
    np.testing.assert_allclose(tp["rh"], t_rh, rtol=1e-12)
