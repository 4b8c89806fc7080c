"""The kick entry point that allocates nothing agrees with the regular mixed kick.

swg_kick_getacch_int_all_tri_pl_noalloc exists for host codes that cannot allocate
device memory while they run: an application that owns every device allocation in its
own fixed pool sized at start-up (an allocation mid-run can fail or fragment the pool),
or one that cannot let cudaMalloc/cudaFree synchronize the device under the work it keeps
in flight on other streams.  It keeps its scratch in one fixed device array that all
calls share, so each case below makes two calls in a row, both into a non-zero acc, and
checks them:

* where the regular entry point swg_kick_getacch_int_all_tri_pl (SWG_MIXED) runs its
  broadcast kernel, the two give the same bits (same kernel, same grid);
* above the size where the regular entry point switches to its symmetric kernel, the two
  agree within the mixed-kick tolerance of the other tests (2e-5 per body, relative);
* every result is within that tolerance of the FP64 oracle.

This file is named to be collected last, so a run that stops at its first failure has
run every other test first.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 2e-5  # mixed-kick tolerance: per-body error relative to |a|


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _relerr(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def _system(seed, npl):
    from swiftest_gb300 import initial_conditions as IC
    cb, pl, _ = IC.make_system(seed=seed, npl=npl, ntp=0)
    return IC.sort_for_integrator(pl, "SYMBA")


@pytest.mark.parametrize("npl,nplm,rad,exact", [
    (3000, 3000, True, True),     # broadcast kernel in both: same bits
    (3000, 3000, False, True),    # norad variant
    (2500, 900, True, True),      # GMTINY loop shape (nplm < npl)
    (20000, 20000, True, False),  # regular entry takes its symmetric kernel here
])
def test_noalloc_kick_matches_regular_entry_point(ctx, npl, nplm, rad, exact):
    torch = pytest.importorskip("torch")
    from swiftest_gb300 import SWG_MIXED, _lib

    lib = _lib.load()
    pl = _system(31 + npl, npl)
    R = pl["radius"] if rad else None
    acc0 = np.random.default_rng(npl).normal(size=(npl, 3)) * 1e-3
    regular = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], R, acc=acc0, nplm=nplm, precision=SWG_MIXED)
    oracle = O.kick_tri_pl(pl["rh"], pl["Gmass"], R, acc=acc0, nplm=nplm)

    dev = torch.device("cuda", 0)
    r = torch.tensor(pl["rh"], dtype=torch.float64, device=dev).contiguous()
    g = torch.tensor(pl["Gmass"], dtype=torch.float64, device=dev).contiguous()
    rd = torch.tensor(R, dtype=torch.float64, device=dev).contiguous() if rad else None
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):  # the second call finds the shared array as the first left it
        acc = torch.tensor(acc0, dtype=torch.float64, device=dev).contiguous()
        rc = lib.swg_kick_getacch_int_all_tri_pl_noalloc(npl, nplm, _dptr(r), _dptr(g), _dptr(rd), _dptr(acc),
                                                         ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        got = acc.cpu().numpy()
        if exact:
            assert np.array_equal(got, regular)
        else:
            assert _relerr(got - acc0, regular - acc0).max() < TOL
        assert _relerr(got - acc0, oracle - acc0).max() < TOL


def test_noalloc_kick_rejects_bad_arguments():
    from swiftest_gb300 import _lib
    lib = _lib.load()
    too_many = 1048576 + 1  # SWG_NOALLOC_MAX_NPL + 1
    assert lib.swg_kick_getacch_int_all_tri_pl_noalloc(too_many, too_many, None, None, None, None, None) == -1
    assert lib.swg_kick_getacch_int_all_tri_pl_noalloc(10, 11, None, None, None, None, None) == -1  # nplm > npl
    assert lib.swg_kick_getacch_int_all_tri_pl_noalloc(10, 10, None, None, None, None, None) == -1  # NULL arrays
