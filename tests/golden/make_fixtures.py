"""Generate tests/golden/solar8.npz from the reference's 8-planet example initial conditions.

Reads examples/Swifter_Swiftest/8pl_0tp/{cb,pl}.swiftest.in of the Swiftest
source tree (ASCII "XV" format: per body a header line "name Gmass rhill",
then radius, position and velocity lines; units AU and days).  Run once where
the reference tree is available:

    python tests/golden/make_fixtures.py /path/to/swiftest
"""
import sys
from pathlib import Path

import numpy as np


def _lines(path):
    return [l.split() for l in Path(path).read_text().splitlines() if l.strip() and not l.startswith("!")]


def main(src):
    d = Path(src) / "examples" / "Swifter_Swiftest" / "8pl_0tp"
    cb = _lines(d / "cb.swiftest.in")
    GMcb, Rcb = float(cb[1][0]), float(cb[2][0])
    pl = _lines(d / "pl.swiftest.in")
    n = int(pl[0][0])
    names, Gm, rhill, rad, rh, vh = [], [], [], [], [], []
    k = 1
    for _ in range(n):
        names.append(pl[k][0])
        Gm.append(float(pl[k][1]))
        rhill.append(float(pl[k][2]))
        rad.append(float(pl[k + 1][0]))
        rh.append([float(x) for x in pl[k + 2][:3]])
        vh.append([float(x) for x in pl[k + 3][:3]])
        k += 4
    out = Path(__file__).with_name("solar8.npz")
    np.savez(out, names=np.array(names), GMcb=GMcb, Rcb=Rcb, Gmass=np.array(Gm), rhill=np.array(rhill),
             radius=np.array(rad), rh=np.array(rh), vh=np.array(vh), dt=1.0)
    print(f"wrote {out}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path to the Swiftest source tree>")
    main(sys.argv[1])
