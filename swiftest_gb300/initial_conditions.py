"""Seeded synthetic planetary systems (no public dataset exists for this path).

Units: AU, solar masses, years, with G = 4 pi^2.  The central body has GM = 4 pi^2
and radius 0.00465 AU.  Draw order per system (numpy ``default_rng(seed)``):
semimajor axis, eccentricity, inclination, node, argument of pericenter, mean
anomaly and mass for massive bodies, then the six elements for test particles.

* masses: log-uniform in [mmin, mmax] (solar masses); radius from a 3 g/cm^3 density
* a ~ U[amin, amax];  e ~ Rayleigh(sigma_e);  i ~ Rayleigh(sigma_i) [rad];  angles ~ U[0, 2 pi)
* Hill radius rhill = a (Gm / (3 GMcb))^(1/3), as swiftest_util_set_rhill
  (src/swiftest/swiftest_util.f90:2260-2280) computes it from the osculating a.

``el2xv`` is the standard two-body conversion (the behaviour of
swiftest_orbel_el2xv, src/swiftest/swiftest_orbel.f90:45-140) written from the
textbook formulae; Kepler's equation is solved by Newton iteration.
"""
from __future__ import annotations

import numpy as np

GU = 4.0 * np.pi ** 2          # G in AU^3 / (Msun yr^2)
GMCB = GU                      # 1 Msun central body
RCB = 0.00465                  # AU
_AU_M = 1.495978707e11
_MSUN_KG = 1.98847e30
RHO_3GCC = 3000.0 * _AU_M ** 3 / _MSUN_KG   # 3 g/cm^3 in Msun / AU^3


def _kepler_E(M, e):
    M = np.mod(M, 2 * np.pi)
    E = np.where(e < 0.8, M, np.pi * np.ones_like(M))
    for _ in range(50):
        f = E - e * np.sin(E) - M
        fp = 1.0 - e * np.cos(E)
        dE = -f / fp
        E = E + dE
        if np.all(np.abs(dE) < 1e-15):
            break
    return E


def el2xv(mu, a, e, inc, capom, omega, capm):
    """Elliptic elements -> heliocentric position/velocity arrays of shape (n, 3)."""
    mu = np.broadcast_to(np.asarray(mu, dtype=np.float64), np.shape(a))
    E = _kepler_E(capm, e)
    cE, sE = np.cos(E), np.sin(E)
    sqe = np.sqrt(1.0 - e * e)
    # perifocal coordinates
    xp = a * (cE - e)
    yp = a * sqe * sE
    n = np.sqrt(mu / a ** 3)
    rr = a * (1.0 - e * cE)
    vxp = -n * a * a * sE / rr
    vyp = n * a * a * sqe * cE / rr
    co, so = np.cos(capom), np.sin(capom)
    cw, sw = np.cos(omega), np.sin(omega)
    ci, si = np.cos(inc), np.sin(inc)
    d11 = cw * co - sw * so * ci
    d12 = cw * so + sw * co * ci
    d13 = sw * si
    d21 = -sw * co - cw * so * ci
    d22 = -sw * so + cw * co * ci
    d23 = cw * si
    r = np.stack([d11 * xp + d21 * yp, d12 * xp + d22 * yp, d13 * xp + d23 * yp], axis=1)
    v = np.stack([d11 * vxp + d21 * vyp, d12 * vxp + d22 * vyp, d13 * vxp + d23 * vyp], axis=1)
    return r, v


def _elements(rng, n, amin, amax, sig_e, sig_i):
    a = rng.uniform(amin, amax, n)
    e = np.minimum(rng.rayleigh(sig_e, n), 0.9)
    inc = rng.rayleigh(sig_i, n)
    capom = rng.uniform(0.0, 2 * np.pi, n)
    omega = rng.uniform(0.0, 2 * np.pi, n)
    capm = rng.uniform(0.0, 2 * np.pi, n)
    return a, e, inc, capom, omega, capm


def make_system(seed=0, npl=100, ntp=1000, mmin=1e-10, mmax=1e-6, amin=0.5, amax=5.0, sig_e=0.01, sig_i=0.005,
                tp_amin=None, tp_amax=None):
    """One seeded system: dicts ``cb``, ``pl`` (rh, vh, Gmass, radius, rhill, mass, a) and ``tp`` (rh, vh)."""
    rng = np.random.default_rng(seed)
    a, e, inc, capom, omega, capm = _elements(rng, npl, amin, amax, sig_e, sig_i)
    mass = np.exp(rng.uniform(np.log(mmin), np.log(mmax), npl))
    Gmass = GU * mass
    rh, vh = el2xv(GMCB + Gmass, a, e, inc, capom, omega, capm) if npl else (np.zeros((0, 3)), np.zeros((0, 3)))
    radius = (3.0 * mass / (4.0 * np.pi * RHO_3GCC)) ** (1.0 / 3.0)
    rhill = a * (Gmass / GMCB / 3.0) ** (1.0 / 3.0)
    ta, te, ti, tO, tw, tM = _elements(rng, ntp, tp_amin or amin, tp_amax or amax, sig_e, sig_i)
    trh, tvh = el2xv(GMCB, ta, te, ti, tO, tw, tM) if ntp else (np.zeros((0, 3)), np.zeros((0, 3)))
    cb = {"Gmass": GMCB, "radius": RCB}
    pl = {"rh": rh, "vh": vh, "Gmass": Gmass, "radius": radius, "rhill": rhill, "mass": mass, "a": a}
    tp = {"rh": trh, "vh": tvh}
    return cb, pl, tp


def sort_for_integrator(pl, integrator):
    """Order massive bodies as the reference's initialise does:
    HELIO/SyMBA by Gmass descending (helio_util.f90:26), WHM by heliocentric
    distance ascending (whm_util.f90:214-215, sort on ir3h descending)."""
    integrator = integrator.upper()
    if integrator in ("HELIO", "SYMBA"):
        order = np.argsort(-pl["Gmass"], kind="stable")
    else:
        order = np.argsort(np.sqrt((pl["rh"] ** 2).sum(axis=1)), kind="stable")
    return {k: (v[order] if isinstance(v, np.ndarray) and len(v) == len(order) else v) for k, v in pl.items()}


# Benchmark configurations (units: AU, Msun, yr)
CONFIGS = {
    # CPU-runnable HELIO case
    "C0": dict(integrator="HELIO", seed=0, npl=100, ntp=1000, mmin=1e-10, mmax=1e-6, amin=0.5, amax=5.0,
               sig_e=0.01, sig_i=0.005, dt=0.01, nsteps=1000, rhscale=6.5),
    # SyMBA, 1-Hill-radius encounter radius
    "C1": dict(integrator="SYMBA", seed=0, npl=2000, ntp=10000, mmin=1e-10, mmax=1e-6, amin=0.3, amax=3.0,
               sig_e=0.01, sig_i=0.005, dt=0.005, nsteps=10000, rhscale=1.0),
}

# Ensemble configurations: system sizes are log-uniform, drawn from default_rng(seed);
# system s is then generated by make_system(seed=s, ...) and sorted for its integrator.
ENSEMBLES = {
    # batched HELIO ensemble: 512 systems, N_pl in [10, 2000], N_tp = 5 N_pl, C0 distributions
    "C3": dict(integrator="HELIO", nsys=512, nmin=10, nmax=2000, tp_per_pl=5, mmin=1e-10, mmax=1e-6, amin=0.5,
               amax=5.0, sig_e=0.01, sig_i=0.005, dt=0.01, rhscale=6.5),
    # batched SyMBA planetesimal disks: 256 systems, N_pl in [500, 5000], no tp
    "C4": dict(integrator="SYMBA", nsys=256, nmin=500, nmax=5000, tp_per_pl=0, mmin=1e-11, mmax=1e-7, amin=0.5,
               amax=2.0, sig_e=0.02, sig_i=0.02, dt=0.002, rhscale=1.0),
}


def ensemble_sizes(nsys, nmin, nmax, seed=0):
    """Per-system massive-body counts, log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), nsys))).astype(np.int32)


def make_ensemble(name="C4", nsys=None, seed=0, scale=1.0, **over):
    """CSR-packed ensemble of independent systems.

    Returns a dict: ``integrator``, ``dt``, ``rhscale``, per-system ``npl``/``ntp``
    (int32) and ``GMcb``/``Rcb``, and the concatenated body arrays ``pl`` (rh, vh,
    Gmass, radius, rhill) and ``tp`` (rh, vh), each system's block sorted for the
    integrator.  ``nsys`` takes the first systems of the configuration; ``scale``
    multiplies every system size (for small test ensembles)."""
    cfg = dict(ENSEMBLES[name])
    cfg.update(over)
    n_all = ensemble_sizes(cfg["nsys"], cfg["nmin"], cfg["nmax"], seed)
    nsys = cfg["nsys"] if nsys is None else int(nsys)
    npl = np.maximum(np.rint(n_all[:nsys] * scale).astype(np.int32), 2 if cfg["integrator"] == "SYMBA" else 1)
    ntp = (npl * cfg["tp_per_pl"]).astype(np.int32)
    pls, tps = [], []
    for s in range(nsys):
        _, pl, tp = make_system(seed=s, npl=int(npl[s]), ntp=int(ntp[s]), mmin=cfg["mmin"], mmax=cfg["mmax"],
                                amin=cfg["amin"], amax=cfg["amax"], sig_e=cfg["sig_e"], sig_i=cfg["sig_i"])
        pls.append(sort_for_integrator(pl, cfg["integrator"]))
        tps.append(tp)
    keys = ("rh", "vh", "Gmass", "radius", "rhill")
    pl = {k: np.concatenate([p[k] for p in pls]) for k in keys}
    tp = {k: (np.concatenate([t[k] for t in tps]) if ntp.sum() else np.zeros((0, 3))) for k in ("rh", "vh")}
    return {"name": name, "integrator": cfg["integrator"], "dt": cfg["dt"], "rhscale": cfg["rhscale"],
            "npl": npl, "ntp": ntp, "GMcb": np.full(nsys, GMCB), "Rcb": np.full(nsys, RCB), "pl": pl, "tp": tp,
            "systems": [(pls[s], tps[s]) for s in range(nsys)]}
