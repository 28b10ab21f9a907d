"""Parity harness shared by the GPU tests, __graft_entry__.smoke() and
bench.py: runs the GPU timestep and the CPU oracle on identical forcing and
summarises the per-field differences."""
from __future__ import annotations

import numpy as np

import oracle_lib as O

# GPU diag-field name -> oracle diag name, for the fields compared
DIAG_MAP = {
    "fe_d": "fe", "fh_d": "fh", "fev": "fev", "fhv": "fhv", "fhs": "fhs", "fns": "fns", "fnv": "fnv", "ga_d": "ga",
    "tv_d": "tv", "tscrn": "tscrn", "qscrn": "qscrn", "rnet_d": "rnet", "us": "us", "cduv": "cduv", "cdtq": "cdtq",
    "fes": "fes", "fevc": "fevc", "fevw": "fevw", "fpn": "fpn", "frday_d": "frday", "fgpp_d": "fgpp",
    "fnpp": "fnpp", "fnee": "fnee", "frp": "frp", "frs": "frs", "trad_d": "trad", "albedo_vis": "albedo_vis",
    "albedo_nir": "albedo_nir", "transd": "transd", "precis": "precis", "through": "through", "fwet": "fwet",
    "wetfac": "wetfac", "potev": "potev", "runoff": "runoff", "ghflux": "ghflux", "sghflux": "sghflux",
    "drybal": "drybal", "wetbal": "wetbal", "ebal": "ebal", "wbal": "wbal", "qssabs": "qssabs", "rniso": "rniso",
    "vlaiw_d": "vlaiw", "tvair": "tvair", "qvair": "qvair", "swnet": "swnet", "lwnet": "lwnet", "wbtot": "wbtot",
    "gswx_sun": "gswx_sun", "gswx_shd": "gswx_shd", "fwsoil": "fwsoil", "dryleaf_passes": "dryleaf_passes",
    "delwc": "delwc", "cls": "cls", "frpw": "frpw", "frpr": "frpr", "rnof1": "rnof1", "rnof2": "rnof2",
    "smelt": "smelt",
}
STATE_FIELDS = ["wb", "wbice", "tgg", "tggsn", "ssdn", "smass", "sdepth", "snowd", "ssdnn", "snage", "pudsto",
                "owetfac", "rtsoil", "tss", "cansto", "cplant", "csoil", "owb", "ebal_tot", "wbal_tot"]

# Tolerances of the spec: fluxes 1e-3 relative with a 1 W/m2 floor,
# temperatures 0.01 K, soil moisture 1e-5 m3/m3.  The carbon fluxes (gross
# primary production fgpp = -fpn + frday, cbl_model_driver_offline.F90:224;
# net photosynthesis fpn and leaf respiration frday, cbl_dryLeaf.F90:659-661)
# are fluxes too, in g C/m2/s: 1e-3 relative with a floor of 1e-7 g C/m2/s
# (0.008 umol CO2/m2/s, 0.03 % of a midday canopy GPP of 3.7e-4).
FLUX_FIELDS = {"fe_d", "fh_d", "fev", "fhv", "fhs", "fns", "fnv", "ga_d", "rnet_d", "fes", "fevc", "fevw", "swnet",
               "lwnet", "qssabs", "rniso"}
CARBON_FLUX_FIELDS = {"fgpp_d", "fpn", "frday_d", "fgpp", "frday", "frpw", "frpr", "frp", "frs", "fnpp", "fnee"}
CARBON_FLUX_FLOOR = 1e-7
TEMP_FIELDS = {"tv_d", "trad_d", "tgg", "tggsn", "tss", "tvair", "tscrn"}
MOIST_FIELDS = {"wb", "wbice"}
# water amounts of one step (mm = kg/m2): runoff and its surface / drainage
# parts, snow melt, canopy water change, throughfall and precipitation
# reaching the soil, the canopy store; 1e-3 relative with a 1e-3 mm floor
WATER_FIELDS = {"runoff", "rnof1", "rnof2", "smelt", "delwc", "precis", "through", "cansto"}
WATER_FLOOR = 1e-3
# screen specific humidity (kg/kg): 1e-3 relative with a 1e-6 floor
HUMID_FIELDS = {"qscrn", "qvair"}


def tolerance(name, ref):
    ref = np.abs(np.asarray(ref, np.float64))
    if name in FLUX_FIELDS:
        return np.maximum(1e-3 * ref, 1.0)
    if name in CARBON_FLUX_FIELDS:
        return np.maximum(1e-3 * ref, CARBON_FLUX_FLOOR)
    if name in WATER_FIELDS:
        return np.maximum(1e-3 * ref, WATER_FLOOR)
    if name in HUMID_FIELDS:
        return np.maximum(1e-3 * ref, 1e-6)
    if name in TEMP_FIELDS:
        return np.full(ref.shape, 0.01)
    if name in MOIST_FIELDS:
        return np.full(ref.shape, 1e-5)
    return None


# An error beyond FLIP x the tolerance is a tile whose iteration took another
# branch (dryLeaf pass count, snow layering, the chaotic Monin-Obukhov tiles),
# not arithmetic noise of the path it shares with the oracle.
FLIP = 10.0


def compare(name, gpu, ref):
    """max and RMS error; with a tolerance also the fraction and count of
    values within it, and the RMS of the errors below FLIP x tolerance
    measured in units of each value's tolerance (rmsn_core)."""
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    e = gpu - ref
    out = {"max": float(np.abs(e).max()) if e.size else 0.0, "rms": float(np.sqrt(np.mean(e * e))) if e.size else 0.0}
    tol = tolerance(name, ref)
    if tol is not None:
        ae = np.abs(e)
        within = ae <= tol
        out["frac_within"] = float(within.mean())
        out["n"] = int(e.size)
        out["n_out"] = int(e.size - within.sum())
        core = ae <= FLIP * tol
        out["rmsn_core"] = float(np.sqrt(np.mean((e[core] / tol[core]) ** 2))) if core.any() else 0.0
        # the field's scalar tolerance (fluxes: the 1 W/m2 floor)
        out["tol"] = float(np.min(tol))
    return out


# Values out of tolerance the GPU may have per value of the reference's own
# FP32 build: the GPU computes the whole canopy, photosynthesis included, in
# FP32 (the reference's REAL build keeps photosynthesis in FP64), and it
# flips branches about 2.6-2.8 times as often as that build on the gridded
# workload at full size (1e6 tiles x 48 steps).
FLIP_RATIO = 3.0


def noise_criterion(g, m):
    """The criterion of a gridded comparison against the FP64 oracle, given
    the GPU's comparison g and the reference's own REAL = FP32 / r_2 = FP64
    build's comparison m on the same inputs (compare() results): the GPU's
    values out of tolerance number at most FLIP_RATIO times that build's, or
    that build's plus 0.1 % of the values (plus 2), and the RMS of its
    errors that did not flip to another branch (below FLIP x tolerance),
    in units of each value's tolerance, is at most 1.  Returns the list of
    failed conditions (empty: passed)."""
    bad = []
    allowed = int(max(FLIP_RATIO * m["n_out"], m["n_out"] + 1e-3 * g["n"])) + 2
    if g["n_out"] > allowed:
        bad.append("out of tolerance: %d values, the FP32 build %d (%d allowed)" % (g["n_out"], m["n_out"], allowed))
    if g["rmsn_core"] > 1.0:
        bad.append("RMS of the unflipped errors %.3g tolerances" % g["rmsn_core"])
    return bad


def run_pair(ts, nsteps, ktau0=1, diag=True, host_forcing=False, precision=0, **switches):
    """Advance the GPU and the oracle ``nsteps`` from a cold start on
    identical forcing.  Returns (gpu_state, gpu_diag, oracle_state, oracle_diag,
    forcing [nsteps, 13, mp])."""
    from cable_gb300 import runtime as R
    g = R.from_tileset(ts)
    g.set_options(diag=diag, capture_forcing=not host_forcing, **switches)
    forc = []
    if host_forcing:
        F = O.forcing(ts, ktau0 - 1, nsteps)
    for n in range(nsteps):
        if host_forcing:
            g.set_forcing(F[n])
        g.step(ktau0 + n, ts.dels)
        if not host_forcing:
            forc.append(g.get("forcing"))
    g.synchronize()
    if not host_forcing:
        F = np.stack(forc)
    gstate = {k: g.get(k) for k in STATE_FIELDS + ["flags"]}
    gdiag = {k: g.get(k)[0] for k in DIAG_MAP} if diag else {}
    g.close()
    st = O.init_state(ts, precision)
    od = O.run(ts, st, nsteps, ktau0=ktau0, forcing=F, precision=precision, **switches)
    ostate = O.split_state(st)
    return gstate, gdiag, ostate, od, F


def parity_report(gstate, gdiag, ostate, odiag):
    rep = {}
    for k in STATE_FIELDS:
        og = ostate["gammzz"] if k == "gammzz1" else ostate[k]
        rep[k] = compare(k, gstate[k], og[: gstate[k].shape[0]])
    for gk, ok in DIAG_MAP.items():
        if gk in gdiag:
            rep[gk] = compare(gk, gdiag[gk], odiag[ok])
    return rep
