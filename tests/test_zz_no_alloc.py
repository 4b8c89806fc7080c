"""The kick entry point that allocates nothing agrees with the regular mixed kick.

swg_kick_getacch_int_all_tri_pl_noalloc exists for host codes that cannot allocate
device memory while they run: an integrator recorded into a CUDA graph (cudaMalloc and
cudaFree are not allowed during stream capture and can synchronize the device) or an
application that owns every device allocation in its own fixed pool.  It keeps its
scratch in one fixed device array that all calls share, so the check runs two calls in
a row and compares each with swg_kick_getacch_int_all_tri_pl (SWG_MIXED) on the same
inputs, within the mixed-kick tolerance used by the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_kick_matches_regular_entry_point(ctx):
    torch = pytest.importorskip("torch")
    from swiftest_gb300 import SWG_MIXED, _lib
    from swiftest_gb300 import initial_conditions as IC

    lib = _lib.load()
    npl = 3000
    cb, pl, _ = IC.make_system(seed=31, npl=npl, ntp=0)
    pl = IC.sort_for_integrator(pl, "SYMBA")
    expected = ctx.kick_getacch_int_all_tri_pl(pl["rh"], pl["Gmass"], pl["radius"], precision=SWG_MIXED)

    dev = torch.device("cuda", 0)
    r = torch.tensor(pl["rh"], dtype=torch.float64, device=dev).contiguous()
    g = torch.tensor(pl["Gmass"], dtype=torch.float64, device=dev).contiguous()
    rad = torch.tensor(pl["radius"], dtype=torch.float64, device=dev).contiguous()
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):
        acc = torch.zeros((npl, 3), dtype=torch.float64, device=dev)
        rc = lib.swg_kick_getacch_int_all_tri_pl_noalloc(npl, npl, _dptr(r), _dptr(g), _dptr(rad), _dptr(acc),
                                                         ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        got = acc.cpu().numpy()
        # mixed-kick tolerance of the other tests: 2e-5 per-body relative error
        rel = np.linalg.norm(got - expected, axis=1) / np.linalg.norm(expected, axis=1)
        assert rel.max() < 2e-5, rel.max()


def test_noalloc_kick_rejects_oversized_input():
    from swiftest_gb300 import _lib
    lib = _lib.load()
    too_many = 1048576 + 1  # SWG_NOALLOC_MAX_NPL + 1
    assert lib.swg_kick_getacch_int_all_tri_pl_noalloc(too_many, too_many, None, None, None, None, None) == -1
