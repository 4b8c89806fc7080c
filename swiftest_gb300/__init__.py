"""swiftest_gb300 -- GB300 (sm_103a) implementation of Swiftest's integrator hot path.

The compute lives in ``libswiftest_gb300.so`` (CUDA kernels behind the C ABI of
``include/swiftest_gb300.h``); this package holds the build recipe, the ctypes
binding, a numpy-facing host layer and the seeded initial-condition generator.
"""
from . import _lib
from ._lib import (SWG_ENC_SORTSWEEP, SWG_ENC_TRIANGULAR, SWG_FP64, SWG_HELIO, SWG_MIXED, SWG_SYMBA, SWG_WHM,
                   SwiftestGB300Error)

__all__ = ["_lib", "SWG_FP64", "SWG_MIXED", "SWG_ENC_TRIANGULAR", "SWG_ENC_SORTSWEEP", "SWG_WHM", "SWG_HELIO",
           "SWG_SYMBA", "SwiftestGB300Error", "Context", "NBodySystem", "Ensemble"]


def __getattr__(name):
    # the compute classes load the shared library on first use (no fallback)
    if name in ("Context", "NBodySystem", "Ensemble"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
