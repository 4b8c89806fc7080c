"""The C-ABI library builds for sm_103a, loads, and exports every symbol the header declares.

No compute call is made here (no GPU in this test).
"""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"\b(swg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared()
    for must in ("swg_kick_getacch_int_all_tri_pl", "swg_kick_getacch_int_all_flat_pl", "swg_kick_getacch_int_all_tp",
                 "swg_drift_all", "swg_encounter_check_all_plpl", "swg_encounter_check_all_plplm",
                 "swg_encounter_check_all_pltp", "swg_system_step"):
        assert must in names


def test_library_exports_all_declared_symbols():
    from swiftest_gb300 import build as B
    lib_path = B.build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from swiftest_gb300 import _lib
    names = _declared()
    missing = [n for n in names if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from swiftest_gb300 import _lib
    with pytest.raises(ImportError):
        _lib._lib = None
        try:
            _lib.load(tmp_path / "absent.so")
        finally:
            _lib._lib = None


def _prototypes():
    """name -> number of parameters, from the header's prototypes."""
    protos = {}
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(swg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
            args = m.group(2).strip()
            protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return protos


def test_python_binding_argument_counts():
    from swiftest_gb300 import _lib
    protos = _prototypes()
    assert protos
    wrong = {n: (k, len(_lib.SIGNATURES[n][1])) for n, k in protos.items() if len(_lib.SIGNATURES[n][1]) != k}
    assert not wrong, wrong


def _fortran_interfaces():
    """bind(C) name -> number of dummy arguments, from fortran/swiftest_gb300_mod.f90."""
    text = (ROOT / "fortran" / "swiftest_gb300_mod.f90").read_text()
    text = re.sub(r"!.*", "", text)
    text = re.sub(r"&\s*\n\s*", " ", text)  # join continuation lines
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", text):
        args = m.group(2).strip()
        out[m.group(3)] = 0 if not args else args.count(",") + 1
    return out


def test_fortran_module_matches_header():
    """The maintainer's iso_c_binding module (not compiled here: no Fortran compiler) names
    declared entry points only, each with the header's number of arguments."""
    protos = _prototypes()
    fort = _fortran_interfaces()
    assert len(fort) >= 40
    unknown = sorted(n for n in fort if n not in protos)
    assert not unknown, unknown
    wrong = {n: (k, protos[n]) for n, k in fort.items() if protos[n] != k}
    assert not wrong, wrong
