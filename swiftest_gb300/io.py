"""ASCII initial-condition files of the reference (IN_TYPE ASCII), read and written.

Restates the formats read by swiftest_io_read_in_cb (src/swiftest/swiftest_io.f90:3162-3215),
swiftest_io_read_in_body and swiftest_io_read_frame_body (:3117-3375) and the parameter keys
of swiftest_io_param_reader (:2300-2500) that select them:

* param file: ``KEY value`` lines; keys are case-insensitive; ``!`` starts a comment.
* central body (CB_IN): name, Gmass, radius, j2rp2, j4rp4 (one value per line), then with
  ROTATION the principal moments Ip(3) and the rotation vector (degrees per time unit).
* massive bodies (PL_IN): nbody, then per body a line ``name Gmass [rhill]`` (rhill with
  RHILL_PRESENT), a radius line with CHK_CLOSE, two lines of ``rh`` and ``vh`` (IN_FORM XV)
  or of ``a e inc`` and ``capom omega capm`` in degrees (IN_FORM EL), then with ROTATION Ip
  and rot.
* test particles (TP_IN): nbody, then per body a ``name`` line and the two XV or EL lines.

Lines starting with ``!`` (the copyright headers of the reference's example files) are
skipped.  Elements are converted to positions and velocities on the GPU
(``Context.el2xv``, swiftest_orbel_el2xv) with mu = GMcb + Gmass for massive bodies and
GMcb for test particles, as swiftest_orbel_el2xv_vec does after set_mu.  With IN_TYPE
NETCDF_DOUBLE (or NETCDF_FLOAT) the run starts from the last frame of the NC_IN data file
(``swiftest_gb300.netcdf``, the restart path of swiftest_io_netcdf_read_frame_system).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

DEG2RAD = np.pi / 180.0
_TRUE = {"YES", "Y", "T", "TRUE", ".TRUE."}


def _records(path):
    out = []
    for line in Path(path).read_text().splitlines():
        s = line.strip()
        if not s or s.startswith("!"):
            continue
        out.append(s.split())
    return out


def read_param(path) -> dict:
    """KEY -> value string (upper-case keys), as the parameter reader tokenises them."""
    par = {}
    for rec in _records(path):
        par[rec[0].upper()] = " ".join(rec[1:])
    return par


def flag(par: dict, key: str, default=False) -> bool:
    v = par.get(key.upper())
    return default if v is None else v.strip().upper() in _TRUE


def read_cb(path, rotation=False) -> dict:
    r = _records(path)
    cb = {"name": r[0][0], "Gmass": float(r[1][0]), "radius": float(r[2][0]), "j2rp2": float(r[3][0]),
          "j4rp4": float(r[4][0])}
    if rotation:
        cb["Ip"] = np.array([float(x) for x in r[5][:3]])
        cb["rot"] = np.array([float(x) for x in r[6][:3]]) * DEG2RAD
    return cb


def read_bodies(path, kind="pl", in_form="XV", rhill_present=False, lclose=False, rotation=False) -> dict:
    """Bodies of a PL_IN / TP_IN file: names and, for massive bodies, Gmass, radius and rhill
    (when present), then rh, vh (XV) or a, e, inc, capom, omega, capm in radians (EL)."""
    if in_form not in ("XV", "EL"):
        raise ValueError(f"{in_form} is not a recognized format code for input files")
    r = _records(path)
    n = int(r[0][0])
    k = 1
    names, Gm, rhill, radius, c1, c2, Ip, rot = [], [], [], [], [], [], [], []
    for _ in range(n):
        names.append(r[k][0])
        if kind == "pl":
            Gm.append(float(r[k][1]))
            if rhill_present:
                rhill.append(float(r[k][2]))
            k += 1
            if lclose:
                radius.append(float(r[k][0]))
                k += 1
        else:
            k += 1
        c1.append([float(x) for x in r[k][:3]])
        c2.append([float(x) for x in r[k + 1][:3]])
        k += 2
        if kind == "pl" and rotation:
            Ip.append([float(x) for x in r[k][:3]])
            rot.append([float(x) * DEG2RAD for x in r[k + 1][:3]])
            k += 2
    out = {"name": np.array(names)}
    if kind == "pl":
        out["Gmass"] = np.array(Gm)
        if rhill_present:
            out["rhill"] = np.array(rhill)
        if lclose:
            out["radius"] = np.array(radius)
        if rotation:
            out["Ip"], out["rot"] = np.array(Ip), np.array(rot)
    c1, c2 = np.array(c1).reshape(-1, 3), np.array(c2).reshape(-1, 3)
    if in_form == "XV":
        out["rh"], out["vh"] = c1, c2
    else:
        out["a"], out["e"], out["inc"] = c1[:, 0], c1[:, 1], c1[:, 2] * DEG2RAD
        out["capom"], out["omega"], out["capm"] = c2[:, 0] * DEG2RAD, c2[:, 1] * DEG2RAD, c2[:, 2] * DEG2RAD
    return out


def el_to_xv(ctx, bodies: dict, GMcb: float) -> dict:
    """rh, vh of element-form bodies (swiftest_orbel_el2xv_vec on the GPU)."""
    mu = GMcb + bodies["Gmass"] if "Gmass" in bodies else np.full(len(bodies["a"]), GMcb)
    rh, vh = ctx.el2xv(mu, bodies["a"], bodies["e"], bodies["inc"], bodies["capom"], bodies["omega"],
                       bodies["capm"])
    out = dict(bodies)
    out["rh"], out["vh"] = rh, vh
    return out


def load_run(param_path, ctx=None) -> dict:
    """The central body, massive bodies and test particles of an ASCII run, positions and
    velocities heliocentric (elements converted with ``ctx``, a ``Context``, for IN_FORM EL).
    Returns {"param", "cb", "pl", "tp"}; massive bodies without RHILL_PRESENT get no rhill."""
    par = read_param(param_path)
    base = Path(param_path).parent
    in_type = par.get("IN_TYPE", "ASCII").upper()
    if in_type in ("NETCDF_DOUBLE", "NETCDF_FLOAT"):
        from . import netcdf
        fr = netcdf.read_frame(base / par.get("NC_IN", "init_cond.nc"))
        return {"param": par, "cb": fr["cb"], "pl": fr["pl"], "tp": fr["tp"] if len(fr["tp"]["rh"]) else None,
                "time": fr["time"]}
    if in_type != "ASCII":
        raise ValueError(f"IN_TYPE {in_type}: ASCII, NETCDF_DOUBLE or NETCDF_FLOAT")
    form = par.get("IN_FORM", "XV").upper()
    rot = flag(par, "ROTATION")
    cb = read_cb(base / par["CB_IN"], rotation=rot)
    pl = read_bodies(base / par["PL_IN"], "pl", form, flag(par, "RHILL_PRESENT"), flag(par, "CHK_CLOSE"), rot)
    tp = read_bodies(base / par["TP_IN"], "tp", form) if "TP_IN" in par and (base / par["TP_IN"]).exists() else None
    if form == "EL":
        if ctx is None:
            raise ValueError("IN_FORM EL needs a Context to convert the elements")
        pl = el_to_xv(ctx, pl, cb["Gmass"])
        if tp is not None:
            tp = el_to_xv(ctx, tp, cb["Gmass"])
    return {"param": par, "cb": cb, "pl": pl, "tp": tp}


def _fmt(x):
    return repr(float(x))


def write_cb(path, cb: dict, rotation=False):
    lines = [cb.get("name", "CB"), _fmt(cb["Gmass"]), _fmt(cb["radius"]), _fmt(cb.get("j2rp2", 0.0)),
             _fmt(cb.get("j4rp4", 0.0))]
    if rotation:
        lines.append(" ".join(_fmt(x) for x in cb["Ip"]))
        lines.append(" ".join(_fmt(x / DEG2RAD) for x in cb["rot"]))
    Path(path).write_text("\n".join(lines) + "\n")


def write_bodies(path, bodies: dict, kind="pl", rhill_present=False, lclose=False):
    """A PL_IN / TP_IN file in XV form (values written to full double precision)."""
    rh, vh = np.asarray(bodies["rh"]).reshape(-1, 3), np.asarray(bodies["vh"]).reshape(-1, 3)
    n = len(rh)
    names = bodies.get("name", [f"{kind}{i + 1}" for i in range(n)])
    lines = [str(n)]
    for i in range(n):
        if kind == "pl":
            head = f"{names[i]} {_fmt(bodies['Gmass'][i])}"
            if rhill_present:
                head += f" {_fmt(bodies['rhill'][i])}"
            lines.append(head)
            if lclose:
                lines.append(_fmt(bodies["radius"][i]))
        else:
            lines.append(str(names[i]))
        lines.append(" ".join(_fmt(x) for x in rh[i]))
        lines.append(" ".join(_fmt(x) for x in vh[i]))
    Path(path).write_text("\n".join(lines) + "\n")
