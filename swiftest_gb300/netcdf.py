"""Output frames and restart of the reference's NetCDF data file (data.nc), NetCDF classic format.

Restates the layout that swiftest_io_netcdf_initialize_output defines
(src/swiftest/swiftest_io.f90:821-1000; names in src/netcdf_io/netcdf_io_module.f90:32-144) and
that swiftest_io_netcdf_write_frame_system / _hdr_system / _cb / _body fill
(swiftest_io.f90:1837-2122), and the restart read of swiftest_io_netcdf_read_frame_system with
the body selection of swiftest_io_netcdf_get_valid_masks (:1190-1279):

* dimensions ``time`` (unlimited), ``space`` (3, labels x y z), ``name`` (one slot per body:
  the central body, the massive bodies, then the test particles, in id order) and ``string32``;
* per body: ``name``, ``id`` (0 for the central body), ``particle_type`` ("Central Body",
  "Massive Body", "Semi-Interacting Massive Body" below GMTINY, "Test Particle");
* per frame: ``time``, ``npl``, ``ntp`` (active bodies), ``nplm`` (with GMTINY), ``status``,
  ``rh`` and ``vh`` (OUT_FORM XV or XVEL), the orbital elements ``a e inc capom omega capm varpi
  lam f cape`` (EL or XVEL; angles in degrees, cape holds the hyperbolic anomaly when e > 1, as
  the reference writes them), ``Gmass``, ``mass`` (Gmass / GU), ``rhill``, ``radius``,
  ``j2rp2``/``j4rp4`` of the central body, and with energies ``KE_orb KE_spin PE BE TE L_orbit
  L_spin L_escape E_collisions E_untracked GMescape``.

On reading a frame, a body is valid when its status is not INACTIVE; valid bodies with Gmass > 0
are massive bodies (slot 0 is the central body), the others test particles.

The reference writes NetCDF-4 (HDF5) through NetCDF-Fortran, whose second unlimited dimension
(``name``) needs that format.  This build has no NetCDF or HDF5 library: the file is NetCDF
classic with 64-bit offsets, written and read with ``scipy.io.netcdf_file``, and ``name`` is a
fixed dimension holding every body of the run (bodies removed by merges or discards keep their
slot with status INACTIVE, as the reference keeps their id slot).  NetCDF readers (xarray,
netCDF4, ncdump) read both formats.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GU_AU_MSUN_YR = 4.0 * np.pi ** 2  # G in AU^3 / (Msun yr^2)
RAD2DEG = 180.0 / np.pi
NAMELEN = 32
INACTIVE = 1  # body status of a removed body (swiftest_globals: INACTIVE)
CB_TYPE, PL_TYPE, PL_TINY_TYPE, TP_TYPE = "Central Body", "Massive Body", "Semi-Interacting Massive Body", \
    "Test Particle"
ELEMENTS = ("a", "e", "inc", "capom", "omega", "capm", "varpi", "lam", "f", "cape")
ENERGY = ("KE_orb", "KE_spin", "PE", "BE", "TE", "E_collisions", "E_untracked", "GMescape")
VECTORS = ("L_orbit", "L_spin", "L_escape")


def _netcdf():
    try:
        from scipy.io import netcdf_file
    except ImportError as e:  # pragma: no cover - scipy is a dependency of the I/O layer
        raise ImportError("NetCDF frames need scipy (scipy.io.netcdf_file)") from e
    return netcdf_file


def _chars(strings, n):
    out = np.full((len(strings), n), b" ", dtype="S1")
    for i, s in enumerate(strings):
        b = str(s).encode()[:n]
        out[i, :len(b)] = np.frombuffer(b, dtype="S1")
    return out


def _strings(chars):
    return [b"".join(row).decode().strip() for row in np.asarray(chars)]


class NetCDFOutput:
    """A data file of output frames (the reference's BIN_OUT with OUT_TYPE NETCDF_DOUBLE).

    ``cb``: the central body dict (name, Gmass, radius, j2rp2, j4rp4); ``npl``/``ntp``: the
    run's body counts (slots of the ``name`` dimension); ``pl_names``/``tp_names``: optional
    names (default ``"pl<i>"``/``"tp<i>"``).  ``out_form``: "XV", "EL" or "XVEL"; ``gmtiny``:
    the GMTINY threshold (0: none); ``lenergy``: write the energy and momentum variables;
    ``GU``: the gravitational constant of the run's units (mass = Gmass / GU)."""

    def __init__(self, path, cb: dict, npl: int, ntp: int, pl_names=None, tp_names=None, out_form="XVEL",
                 gmtiny=0.0, lenergy=True, GU=GU_AU_MSUN_YR):
        netcdf_file = _netcdf()
        self.path = Path(path)
        self.cb, self.npl, self.ntp = cb, int(npl), int(ntp)
        self.out_form = out_form.upper()
        if self.out_form not in ("XV", "EL", "XVEL"):
            raise ValueError(f"out_form {out_form!r}: XV, EL or XVEL")
        self.gmtiny, self.lenergy, self.GU = float(gmtiny), bool(lenergy), float(GU)
        n = 1 + self.npl + self.ntp
        f = netcdf_file(str(self.path), "w", version=2)
        f.createDimension("time", None)
        f.createDimension("space", 3)
        f.createDimension("name", n)
        f.createDimension("string32", NAMELEN)
        f.createVariable("time", "d", ("time",))
        f.createVariable("space", "c", ("space",))[:] = np.array([b"x", b"y", b"z"])
        names = [cb.get("name", "Sun")] + list(pl_names if pl_names is not None else
                                                 [f"pl{i + 1}" for i in range(self.npl)])
        names += list(tp_names if tp_names is not None else [f"tp{i + 1}" for i in range(self.ntp)])
        f.createVariable("name", "c", ("name", "string32"))[:] = _chars(names, NAMELEN)
        f.createVariable("id", "i", ("name",))[:] = np.arange(n, dtype=np.int32)
        f.createVariable("particle_type", "c", ("name", "string32"))
        self._types = None
        for v in ("status",):
            f.createVariable(v, "i", ("time", "name"))
        for v in ("npl", "ntp") + (("nplm",) if self.gmtiny > 0 else ()):
            f.createVariable(v, "i", ("time",))
        if self.out_form in ("XV", "XVEL"):
            for v in ("rh", "vh"):
                f.createVariable(v, "d", ("time", "name", "space"))
        if self.out_form in ("EL", "XVEL"):
            for v in ELEMENTS:
                f.createVariable(v, "d", ("time", "name"))
        for v in ("Gmass", "mass", "rhill", "radius"):
            f.createVariable(v, "d", ("time", "name"))
        for v in ("j2rp2", "j4rp4"):
            f.createVariable(v, "d", ("time",))
        if self.lenergy:
            for v in ENERGY:
                f.createVariable(v, "d", ("time",))
            for v in VECTORS:
                f.createVariable(v, "d", ("time", "space"))
        self.f = f
        self.tslot = 0

    def write_frame(self, t, system, ctx=None):
        """Append the state of ``system`` (an ``NBodySystem``) at time ``t`` as the next frame.
        ``ctx`` (a ``Context``) converts to orbital elements on the GPU (needed for EL/XVEL)."""
        rh, vh, st = system.get_pl()
        Gm, R, rhill = system.get_pl_masses()
        if self.ntp:
            trh, tvh, tst = system.get_tp()
        else:
            trh = tvh = np.zeros((0, 3))
            tst = np.zeros(0, np.int32)
        frame = {"rh": rh, "vh": vh, "status": st, "Gmass": Gm, "radius": R, "rhill": rhill, "trh": trh,
                 "tvh": tvh, "tstatus": tst}
        if self.lenergy:
            frame["energy"] = system.energy()
        self.write_arrays(t, frame, ctx if ctx is not None else getattr(system, "ctx", None))

    def write_arrays(self, t, fr: dict, ctx=None):
        """Append a frame from host arrays: rh, vh, status, Gmass, radius, rhill of the massive
        bodies, trh, tvh, tstatus of the test particles, and optionally ``energy`` (the dict of
        ``NBodySystem.energy``)."""
        f, k = self.f, self.tslot
        cb, npl, ntp = self.cb, self.npl, self.ntp
        GMcb = float(cb["Gmass"])
        Gm = np.asarray(fr["Gmass"], dtype=float)
        st = np.concatenate([[0], np.asarray(fr["status"]), np.asarray(fr["tstatus"])]).astype(np.int32)
        f.variables["time"][k] = float(t)
        f.variables["status"][k] = st
        f.variables["npl"][k] = int(np.sum(np.asarray(fr["status"]) != INACTIVE))
        f.variables["ntp"][k] = int(np.sum(np.asarray(fr["tstatus"]) != INACTIVE))
        if self.gmtiny > 0:
            f.variables["nplm"][k] = int(np.sum((np.asarray(fr["status"]) != INACTIVE) & (Gm > self.gmtiny)))
        if self._types is None:  # particle types from the first frame's masses
            types = [CB_TYPE] + [PL_TINY_TYPE if (self.gmtiny > 0 and g <= self.gmtiny) else PL_TYPE for g in Gm]
            f.variables["particle_type"][:] = _chars(types + [TP_TYPE] * ntp, NAMELEN)
            self._types = types
        rh = np.concatenate([np.zeros((1, 3)), np.reshape(fr["rh"], (npl, 3)), np.reshape(fr["trh"], (ntp, 3))])
        vh = np.concatenate([np.zeros((1, 3)), np.reshape(fr["vh"], (npl, 3)), np.reshape(fr["tvh"], (ntp, 3))])
        if self.out_form in ("XV", "XVEL"):
            f.variables["rh"][k] = rh
            f.variables["vh"][k] = vh
        if self.out_form in ("EL", "XVEL"):
            if ctx is None:
                raise ValueError("orbital elements need a Context (swiftest_orbel_xv2el on the GPU)")
            mu = np.concatenate([GMcb + Gm, np.full(ntp, GMcb)])
            el = ctx.xv2el(mu, rh[1:], vh[1:])
            for v in ELEMENTS:
                x = np.full(1 + npl + ntp, np.nan)
                if v == "cape":
                    x[1:] = np.where(el["e"] < 1.0, el["cape"], np.where(el["e"] > 1.0, el["capf"], np.nan)) * RAD2DEG
                else:
                    x[1:] = el[v] * (RAD2DEG if v not in ("a", "e") else 1.0)
                f.variables[v][k] = x
        f.variables["Gmass"][k] = np.concatenate([[GMcb], Gm, np.zeros(ntp)])
        f.variables["mass"][k] = np.concatenate([[GMcb], Gm, np.zeros(ntp)]) / self.GU
        f.variables["radius"][k] = np.concatenate([[float(cb["radius"])], np.asarray(fr["radius"]), np.zeros(ntp)])
        f.variables["rhill"][k] = np.concatenate([[0.0], np.asarray(fr["rhill"]), np.zeros(ntp)])
        f.variables["j2rp2"][k] = float(cb.get("j2rp2", 0.0))
        f.variables["j4rp4"][k] = float(cb.get("j4rp4", 0.0))
        if self.lenergy and "energy" in fr:
            e = fr["energy"]
            vals = {"KE_orb": e["ke"], "KE_spin": 0.0, "PE": e["pe"], "BE": e["be"], "TE": e["te"],
                    "E_collisions": e.get("E_collisions", 0.0), "E_untracked": 0.0, "GMescape": 0.0}
            for v in ENERGY:
                f.variables[v][k] = float(vals[v])
            f.variables["L_orbit"][k] = np.asarray(e["L"], dtype=float)
            f.variables["L_spin"][k] = np.zeros(3)
            f.variables["L_escape"][k] = np.asarray(e.get("L_escape", np.zeros(3)), dtype=float)
        self.f.flush()
        self.tslot += 1

    def close(self):
        if self.f is not None:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_frame(path, tslot: int = -1) -> dict:
    """One frame of a data file (the last by default), for a restart: {"time", "cb", "pl", "tp",
    "tslot"} with the valid bodies only (status not INACTIVE), massive bodies where Gmass > 0,
    in id order; pl holds rh, vh, Gmass, radius, rhill, name, id; tp rh, vh, name, id."""
    netcdf_file = _netcdf()
    with netcdf_file(str(path), "r", mmap=False) as f:
        nt = f.variables["time"].shape[0]
        k = tslot if tslot >= 0 else nt + tslot
        if not 0 <= k < nt:
            raise IndexError(f"frame {tslot} of {nt}")
        g = lambda v: np.array(f.variables[v][k])  # noqa: E731
        names = _strings(f.variables["name"][:])
        ids = np.array(f.variables["id"][:])
        Gm, st = g("Gmass"), g("status")
        valid = st != INACTIVE
        plm = np.isfinite(Gm) & (Gm > 0.0) & valid
        plm[0] = False
        tpm = ~(np.isfinite(Gm) & (Gm > 0.0)) & valid
        tpm[0] = False
        if "rh" in f.variables:
            rh, vh = g("rh"), g("vh")
        else:
            raise ValueError("frames without rh/vh (OUT_FORM EL) are not read back")
        cb = {"name": names[0], "Gmass": float(Gm[0]), "radius": float(g("radius")[0]),
              "j2rp2": float(g("j2rp2")), "j4rp4": float(g("j4rp4"))}
        pl = {"rh": rh[plm], "vh": vh[plm], "Gmass": Gm[plm], "radius": g("radius")[plm], "rhill": g("rhill")[plm],
              "name": [names[i] for i in np.flatnonzero(plm)], "id": ids[plm]}
        tp = {"rh": rh[tpm], "vh": vh[tpm], "name": [names[i] for i in np.flatnonzero(tpm)], "id": ids[tpm]}
        return {"time": float(f.variables["time"][k]), "cb": cb, "pl": pl, "tp": tp, "tslot": k}
