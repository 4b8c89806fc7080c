"""The oracle's restatement of the reference's perfect-merge resolution (collision_resolve_plpl
with collision_generate_merge, src/collision/collision_resolve.f90:521-662,
collision_generate.f90:158-260), checked through the bookkeeping the reference keeps for it.

A crowded SyMBA disk (radii inflated 300x) merges several times in 200 steps.  Per step:
* energy: the total energy jumps at a merge, and the reference books the jump in
  E_collisions, so te - E_collisions must change at a merge step no more than at the
  steps without one (swiftest_io.f90:181-183);
* angular momentum: the merged body's velocity is torqued to restore the impactors'
  angular momentum about their centre of mass (collision_util_velocity_torque); a velocity
  change at the body's position cannot restore the component along that position, so the
  system's angular momentum changes at a merge, but by less than the internal angular
  momentum the reference books in L_escape, and its component along the total angular
  momentum (the disk normal) stays far below that.
No GPU is used.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swiftest_gb300 import initial_conditions as IC


@pytest.fixture(scope="module")
def history():
    cb, pl, tp = IC.make_system(seed=7, npl=150, ntp=300, amin=0.8, amax=1.2, mmin=1e-9, mmax=1e-6)
    pl = IC.sort_for_integrator(pl, "SYMBA")
    pl["radius"] = pl["radius"] * 300.0
    s = O.OracleSystem("SYMBA", cb, pl, tp, dt=0.005, rhscale=3.0)
    out = [s.energy()]
    for _ in range(200):
        s.step(1)
        out.append(s.energy())
    return out, s.stats()


def test_merges_happen(history):
    h, stats = history
    assert stats["collisions"] > 0
    merges = sum(np.linalg.norm(b["L_escape"] - a["L_escape"]) > 0 for a, b in zip(h, h[1:]))
    assert merges >= 3


def test_energy_minus_collision_energy_is_continuous(history):
    h, _ = history
    E0 = abs(h[0]["te"])
    quiet, merge, booked = [], [], []
    for a, b in zip(h, h[1:]):
        d = abs((b["te"] - b["E_collisions"]) - (a["te"] - a["E_collisions"])) / E0
        if np.linalg.norm(b["L_escape"] - a["L_escape"]) > 0:
            merge.append(d)
            booked.append(abs(b["E_collisions"] - a["E_collisions"]) / E0)
        else:
            quiet.append(d)
    assert max(booked) > 100 * max(quiet)  # the merges do change the energy ...
    assert max(merge) <= 1.5 * max(quiet)  # ... and the booked amount is exactly that change


def test_angular_momentum_through_merges(history):
    h, _ = history
    L0 = np.linalg.norm(h[0]["L"])
    zhat = h[0]["L"] / L0
    for a, b in zip(h, h[1:]):
        esc = np.linalg.norm(b["L_escape"] - a["L_escape"])
        dL = b["L"] - a["L"]
        if esc > 0:
            assert np.linalg.norm(dL) < esc
            assert abs(dL @ zhat) < 0.01 * esc  # the torque restores the part along the disk normal
        else:
            assert np.linalg.norm(dL) < 1e-13 * L0  # no merge: conserved to rounding
