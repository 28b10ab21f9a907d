"""Field-by-field parity of the plain GPU timestep against the FP64 oracle at
the gridded workload's full size: 1,000,000 tiles (PFT U{1..17}, soil
U{1..9}, LAI lognormal clipped to [0.1, 8], per-tile forcing jitter), 48
half-hour steps, diagnostics off, i.e. the kernels the benchmark times.

Every step, the forcing the GPU generated (captured from the in-kernel
generator) drives the oracle twice: in FP64 (the oracle) and in the
reference's own REAL = FP32 / r_2 = FP64 mix (the reference's precision
noise on the same inputs).  For each output row (latent and sensible heat,
GPP, leaf respiration, canopy temperature, net radiation, ground heat flux,
radiative temperature) the max and RMS error over every tile-step and the
fraction of tile-steps within tolerance are accumulated, for the GPU and for
the precision mix; the soil temperature and moisture profiles (per layer),
snow and surface temperature are compared after the last step.

Test infrastructure: runs the oracle as the checker.  Run as
``python tests/parity_full.py --json report.json`` for the report, or through
tests/test_gpu_parity.py::test_config2_full_size_against_fp64_oracle."""
from __future__ import annotations

import time

import numpy as np

import harness as H
import oracle_lib as O

# output rows of the field "out" and their tolerance class (harness names)
OUT_ROWS = [("fe", "fe_d"), ("fh", "fh_d"), ("fgpp", "fgpp_d"), ("frday", "frday_d"), ("tv", "tv_d"),
            ("rnet", "rnet_d"), ("ga", "ga_d"), ("trad", "trad_d")]
UNITS = {"fe": "W/m2", "fh": "W/m2", "fgpp": "g C/m2/s", "frday": "g C/m2/s", "tv": "K", "rnet": "W/m2",
         "ga": "W/m2", "trad": "K", "tgg": "K", "wb": "m3/m3", "wbice": "m3/m3", "tggsn": "K", "tss": "K",
         "snowd": "kg/m2"}
TOL_TEXT = {"flux": "1e-3 relative, floor 1 W/m2", "carbon": "1e-3 relative, floor 1e-7 g C/m2/s",
            "temp": "0.01 K", "moist": "1e-5 m3/m3"}


def _tol_class(hname):
    if hname in H.FLUX_FIELDS:
        return "flux"
    if hname in H.CARBON_FLUX_FIELDS:
        return "carbon"
    if hname in H.TEMP_FIELDS:
        return "temp"
    if hname in H.MOIST_FIELDS:
        return "moist"
    return None


class _Acc:
    """Running max / RMS / within-tolerance count of an error field."""

    def __init__(self):
        self.n = 0
        self.sq = 0.0
        self.mx = 0.0
        self.within = 0
        self.core_n = 0
        self.core_sq = 0.0
        self.nonfinite = 0

    def add(self, err, tol):
        ok = np.isfinite(err)
        self.nonfinite += int(err.size - ok.sum())
        e = np.abs(err[ok])
        self.n += e.size
        self.sq += float(np.sum(e * e))
        self.mx = max(self.mx, float(e.max()) if e.size else 0.0)
        if tol is not None:
            t = tol[ok]
            self.within += int(np.sum(e <= t))
            core = e <= H.FLIP * t
            self.core_n += int(core.sum())
            self.core_sq += float(np.sum((e[core] / t[core]) ** 2))

    def row(self, tol_scalar):
        """The harness.compare statistics of everything added."""
        r = {"max": self.mx, "rms": float(np.sqrt(self.sq / max(1, self.n))), "n": self.n}
        if tol_scalar is not None:
            r["frac_within"] = self.within / max(1, self.n)
            r["n_out"] = self.n - self.within
            r["rmsn_core"] = float(np.sqrt(self.core_sq / max(1, self.core_n)))
            r["tol"] = tol_scalar
        if self.nonfinite:
            r["nonfinite"] = self.nonfinite
        return r


def config2_report(mp=1_000_000, nsteps=48, seed=12345, order=2, device=0, **switches):
    """Runs the comparison and returns {"workload", "fields": {name: {...}},
    "seconds"}.  Field entries: "gpu" and "precision_mix" rows (max, RMS,
    fraction within tolerance), the tolerance and the unit."""
    from cable_gb300 import runtime as R
    from cable_gb300 import workloads as W
    t0 = time.perf_counter()
    ts = W.grid(mp, seed=seed, nsteps=nsteps)
    g = R.from_tileset(ts, device=device, order=order)
    g.set_options(diag=False, capture_forcing=True, **switches)
    st64 = O.init_state(ts, 0)
    st32 = O.init_state(ts, 1)
    acc = {name: (_Acc(), _Acc()) for name, _ in OUT_ROWS}
    t_gpu = t_cpu = 0.0
    for k in range(nsteps):
        a = time.perf_counter()
        g.step(k + 1, ts.dels)
        F = g.get("forcing")[None]
        out = g.get("out").astype(np.float64)
        t_gpu += time.perf_counter() - a
        a = time.perf_counter()
        d64 = O.run(ts, st64, 1, ktau0=k + 1, forcing=F, precision=0, **switches)
        d32 = O.run(ts, st32, 1, ktau0=k + 1, forcing=F, precision=1, **switches)
        t_cpu += time.perf_counter() - a
        for i, (name, hname) in enumerate(OUT_ROWS):
            ref = np.asarray(d64[name], np.float64)
            tol = H.tolerance(hname, ref)
            acc[name][0].add(out[i] - ref, tol)
            acc[name][1].add(np.asarray(d32[name], np.float64) - ref, tol)
    g.synchronize()
    fields = {}
    for name, hname in OUT_ROWS:
        cls = _tol_class(hname)
        tol_scalar = 1.0 if cls == "flux" else (H.CARBON_FLUX_FLOOR if cls == "carbon" else None)
        if cls == "temp":
            tol_scalar = 0.01
        fields[name] = {"unit": UNITS[name], "tolerance": TOL_TEXT[cls], "tol": tol_scalar,
                        "gpu": acc[name][0].row(tol_scalar), "precision_mix": acc[name][1].row(tol_scalar),
                        "over": "every tile-step (%d x %d)" % (mp, nsteps)}
    o64 = O.split_state(st64)
    o32 = O.split_state(st32)
    for name, hname in (("tgg", "tgg"), ("wb", "wb"), ("wbice", "wbice"), ("tggsn", "tggsn"), ("tss", "tss"),
                        ("snowd", "snowd")):
        gv = np.asarray(g.get(name), np.float64)
        nl = gv.shape[0]
        cls = _tol_class(hname)
        tol_scalar = {"temp": 0.01, "moist": 1e-5}.get(cls)
        for layer in range(nl):
            ref = np.asarray(o64[name][layer], np.float64)
            tol = H.tolerance(hname, ref)
            ag, ar = _Acc(), _Acc()
            ag.add(gv[layer] - ref, tol)
            ar.add(np.asarray(o32[name][layer], np.float64) - ref, tol)
            key = name if nl == 1 else "%s[%d]" % (name, layer + 1)
            fields[key] = {"unit": UNITS[name], "tolerance": TOL_TEXT.get(cls, "none stated"), "tol": tol_scalar,
                           "gpu": ag.row(tol_scalar), "precision_mix": ar.row(tol_scalar),
                           "over": "every tile after step %d" % nsteps}
    g.close()
    return {"workload": "grid: %d tiles (PFT U{1..17}, soil U{1..9}, LAI lognormal, forcing jitter), %d steps of "
                        "%g s, tile order %d, diagnostics off" % (mp, nsteps, ts.dels, order),
            "oracle": "FP64 CPU restatement (precision 0); precision_mix = REAL FP32 / r_2 FP64 (precision 1)",
            "switches": switches or "offline defaults", "fields": fields,
            "seconds": {"total": time.perf_counter() - t0, "gpu_steps_and_copies": t_gpu, "oracle": t_cpu}}


def markdown(rep):
    """The report as a markdown table."""
    lines = ["| field | unit | tolerance | GPU max | GPU RMS | GPU RMS unflipped (tolerances) | GPU within | "
             "FP32-mix max | FP32-mix RMS | FP32-mix within | criterion |", "|---|---|---|---|---|---|---|---|---|---|---|"]
    for k, r in rep["fields"].items():
        g, m = r["gpu"], r["precision_mix"]
        fw = lambda x: ("%.5f" % x["frac_within"]) if "frac_within" in x else "-"
        rc = ("%.3g" % g["rmsn_core"]) if "rmsn_core" in g else "-"
        ok = "-" if r["tol"] is None else ("pass" if not H.noise_criterion(g, m) else "FAIL")
        lines.append("| %s | %s | %s | %.3g | %.3g | %s | %s | %.3g | %.3g | %s | %s |" % (
            k, r["unit"], r["tolerance"], g["max"], g["rms"], rc, fw(g), m["max"], m["rms"], fw(m), ok))
    return "\n".join(lines)


if __name__ == "__main__":
    import argparse
    import json
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    ap = argparse.ArgumentParser(description="full-size field-by-field parity report (GPU against the FP64 oracle)")
    ap.add_argument("--mp", type=int, default=1_000_000)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--json", default=None, help="write the report here as JSON")
    a = ap.parse_args()
    rep = config2_report(mp=a.mp, nsteps=a.steps)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(rep, f, indent=1)
    print(markdown(rep))
    print(json.dumps(rep["seconds"]))
