"""ctypes binding of ``libswiftest_gb300.so`` (the C ABI in include/swiftest_gb300.h).

The library is loaded from the package directory.  There is no fallback: if the
shared library is missing the import of the compute entry points raises, so a
missing build can never silently run anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libswiftest_gb300.so"

SWG_OK = 0
SWG_ERR_ARG = -1
SWG_ERR_CUDA = -2
SWG_ERR_CAPACITY = -3
SWG_ERR_NOMEM = -4
SWG_ERR_DRIFT = -5
SWG_ERR_RECURSION = -6
SWG_ERR_STATE = -7
SWG_MEM_HOST = 0
SWG_MEM_DEVICE = 1
SWG_FP64 = 0
SWG_MIXED = 1
SWG_KICK_NVARIANT = 5
SWG_KICK_SYMMETRIC = 5
SWG_ENC_TRIANGULAR = 0
SWG_ENC_SORTSWEEP = 1
SWG_WHM = 0
SWG_HELIO = 1
SWG_SYMBA = 2

_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64
_D = C.c_double
_INT = C.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "swg_create": (_INT, [C.POINTER(_P), _INT]),
    "swg_destroy": (_INT, [_P]),
    "swg_synchronize": (_INT, [_P]),
    "swg_last_error": (C.c_char_p, [_P]),
    "swg_launch_count": (_I64, [_P]),
    "swg_kick_getacch_int_all_tri_pl": (_INT, [_P, _I32, _I32, _P, _P, _P, _P, _INT, _INT]),
    "swg_kick_getacch_int_all_flat_pl": (_INT, [_P, _I32, _I32, _I64, _P, _P, _P, _P, _P, _INT, _INT]),
    "swg_kick_getacch_int_all_tp": (_INT, [_P, _I32, _I32, _P, _P, _P, _P, _P, _INT, _INT]),
    "swg_kick_getacch_int_all_tri_pl_noalloc": (_INT, [_I32, _I32, _P, _P, _P, _P, _P]),
    "swg_orbel_el2xv": (_INT, [_P, _I32] + [_P] * 9 + [_INT]),
    "swg_orbel_xv2el": (_INT, [_P, _I32] + [_P] * 14 + [_INT]),
    "swg_drift_all": (_INT, [_P, _P, _P, _P, _I32, _I32, _D, _D, _P, _P, _INT]),
    "swg_encounter_check_all_plpl": (_INT, [_P, _INT, _I32, _P, _P, _P, _D, _I64, C.POINTER(_I64), _P, _P, _P, _INT]),
    "swg_encounter_check_all_plplm": (_INT, [_P, _INT, _I32, _I32, _P, _P, _P, _P, _P, _P, _D, _I64,
                                             C.POINTER(_I64), _P, _P, _P, _INT]),
    "swg_encounter_check_all_pltp": (_INT, [_P, _INT, _I32, _I32, _P, _P, _P, _P, _P, _D, _I64, C.POINTER(_I64),
                                            _P, _P, _P, _INT]),
    "swg_util_sort_index": (_INT, [_P, _I64, _P, _P, _INT]),
    "swg_system_create": (_INT, [_P, _INT, _I32, _I32, C.POINTER(_P)]),
    "swg_system_destroy": (_INT, [_P]),
    "swg_system_set_cb": (_INT, [_P, _D, _D]),
    "swg_system_set_pl": (_INT, [_P, _P, _P, _P, _P, _P]),
    "swg_system_set_tp": (_INT, [_P, _P, _P]),
    "swg_system_set_param": (_INT, [_P, _D, _INT, _INT, _INT, _D, _INT, _D, _INT]),
    "swg_system_initialize": (_INT, [_P]),
    "swg_system_step": (_INT, [_P, _I32]),
    "swg_system_get_pl": (_INT, [_P, _P, _P, _P]),
    "swg_system_get_pl_masses": (_INT, [_P, _P, _P, _P]),
    "swg_system_get_tp": (_INT, [_P, _P, _P, _P]),
    "swg_system_energy": (_INT, [_P, _P]),
    "swg_system_collision_terms": (_INT, [_P, _P]),
    "swg_system_stats": (_INT, [_P, _P]),
    "swg_system_plpl_list": (_INT, [_P, _I64, C.POINTER(_I64), _P, _P]),
    "swg_system_pltp_list": (_INT, [_P, _I64, C.POINTER(_I64), _P, _P]),
    "swg_system_set_state": (_INT, [_P, _P, _P, _P, _P]),
    "swg_system_get_state_async": (_INT, [_P, _P, _P, _P, _P]),
    "swg_system_profile": (_INT, [_P, _INT]),
    "swg_system_profile_read": (_INT, [_P, _P]),
    "swg_ensemble_create": (_INT, [_P, _INT, _I32, _P, _P, C.POINTER(_P)]),
    "swg_ensemble_destroy": (_INT, [_P]),
    "swg_ensemble_set_cb": (_INT, [_P, _P, _P]),
    "swg_ensemble_set_pl": (_INT, [_P, _P, _P, _P, _P, _P]),
    "swg_ensemble_set_tp": (_INT, [_P, _P, _P]),
    "swg_ensemble_set_param": (_INT, [_P, _D, _D, _INT, _INT]),
    "swg_ensemble_set_encounter_modes": (_INT, [_P, _INT, _INT]),
    "swg_ensemble_initialize": (_INT, [_P]),
    "swg_ensemble_step": (_INT, [_P, _I32]),
    "swg_ensemble_get_pl": (_INT, [_P, _P, _P, _P]),
    "swg_ensemble_get_pl_masses": (_INT, [_P, _P, _P, _P]),
    "swg_ensemble_get_tp": (_INT, [_P, _P, _P, _P]),
    "swg_ensemble_energy": (_INT, [_P, _P]),
    "swg_ensemble_collision_terms": (_INT, [_P, _P]),
    "swg_ensemble_stats": (_INT, [_P, _P]),
    "swg_ensemble_plpl_list": (_INT, [_P, _I32, _I64, C.POINTER(_I64), _P, _P]),
    "swg_ensemble_set_state": (_INT, [_P, _P, _P, _P, _P]),
    "swg_ensemble_get_state_async": (_INT, [_P, _P, _P, _P, _P]),
    "swg_ensemble_use_graphs": (_INT, [_P, _INT]),
    "swg_ensemble_set_kick_variant": (_INT, [_P, _INT]),
    "swg_ensemble_set_kick_strip": (_INT, [_P, _INT]),
    "swg_ensemble_set_kick_warps": (_INT, [_P, _INT]),
    "swg_ensemble_set_kick_tile": (_INT, [_P, _INT]),
    "swg_system_reset_first_step": (_INT, [_P]),
    "swg_ensemble_reset_first_step": (_INT, [_P]),
    "swg_ensemble_set_kick_group": (_INT, [_P, _INT]),
    "swg_ensemble_set_gmtiny": (_INT, [_P, C.c_double]),
    "swg_ensemble_kick_variant": (_INT, [_P, _INT, C.POINTER(_INT)]),
    "swg_ensemble_getacch_int_pl": (_INT, [_P, _P]),
    "swg_ensemble_profile": (_INT, [_P, _INT]),
    "swg_ensemble_profile_read": (_INT, [_P, _P]),
    "swg_flush_l2": (_INT, [_P, _I64]),
    "swg_event_record": (_INT, [_P, _INT]),
    "swg_event_elapsed": (_INT, [_P, _INT, _INT, C.POINTER(_D)]),
    "swg_probe_peak": (_INT, [_P, _INT, C.POINTER(_D)]),
}

_lib = None


class SwiftestGB300Error(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn: str, code: int, msg: str = ""):
        super().__init__(f"{fn} failed with status {code}{': ' + msg if msg else ''}")
        self.code = code


def load(path: Path | None = None) -> C.CDLL:
    """Load the shared library (once) and attach the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(swiftest_gb300 has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
