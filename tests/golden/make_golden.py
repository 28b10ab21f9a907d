"""Writes the golden fixtures under tests/golden/ from the FP64 oracle.

The reference's own tests hold no golden vectors for cbm() (its unit tests
cover netCDF I/O only, tests/test_cable_netcdf.F90), and the reference
Fortran cannot be compiled here, so these fixtures record the FP64 CPU
restatement (oracle/cbm_ref.hpp, precision 0) on seeded synthetic inputs.
They serve two purposes: the CPU tests re-run the oracle against them (any
change to the oracle's physics shows up as a fixture mismatch), and the GPU
tests compare the CUDA timestep with them, with the committed forcing fed
through the host-forcing path, so the GPU check does not depend on the
oracle library being buildable on the GPU host.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_lib as O  # noqa: E402
from cable_gb300 import workloads as W  # noqa: E402

# Diagnostics recorded for every step of the site case, final step of the
# gridded cases (oracle names).
DIAG = ["fe", "fh", "fev", "fes", "fevc", "ga", "tv", "rnet", "fgpp", "frday", "trad", "ebal", "wbal", "drybal",
        "dryleaf_passes", "runoff", "ghflux"]
STATE = ["wb", "wbice", "tgg", "tggsn", "ssdn", "smass", "sdepth", "snowd", "ssdnn", "snage", "cansto", "tss",
         "rtsoil", "owetfac", "pudsto", "cplant", "csoil", "owb", "ebal_tot", "wbal_tot", "isflag"]
TILE = ["iveg", "isoilm", "vlai", "lat", "lonphase", "tbase", "swscale", "snowd0", "tgg0", "wb0"]

CASES = {
    # name: (tileset, steps, per-step diagnostics and full forcing)
    "site5": (lambda: W.site5(nsteps=96), 96, True),
    "grid128": (lambda: W.grid(mp=128, seed=777, nsteps=48), 48, False),
    "snow128": (lambda: W.snow_grid(mp=128, seed=4242, nsteps=48), 48, False),
}


def make_case(name):
    mk, nsteps, per_step = CASES[name]
    ts = mk()
    F = O.forcing(ts, 0, nsteps)
    st = O.init_state(ts, 0)
    steps = []
    mix = None
    if per_step:
        # the same run in the reference's own precision mix (REAL = FP32,
        # r_2 = FP64): its distance from the FP64 run is the reference's
        # precision noise, the floor any FP32 implementation is held to
        st32 = O.init_state(ts, 1)
        steps32 = []
        for n in range(nsteps):
            d = O.run(ts, st, 1, ktau0=1 + n, forcing=F[n:n + 1], precision=0, nthreads=1)
            steps.append(np.stack([d[k] for k in DIAG]))
            d = O.run(ts, st32, 1, ktau0=1 + n, forcing=F[n:n + 1], precision=1, nthreads=1)
            steps32.append(np.stack([d[k] for k in DIAG]))
        diag = np.stack(steps)                      # [nsteps, ndiag, mp]
        mix = np.stack(steps32)
    else:
        d = O.run(ts, st, nsteps, ktau0=1, forcing=F, precision=0, nthreads=1)
        diag = np.stack([d[k] for k in DIAG])[None]  # [1, ndiag, mp]
    s = O.split_state(st)
    # The site case keeps its whole forcing (fed to the GPU through the host
    # path); the gridded cases keep the last step's forcing only and are run
    # on the GPU from its in-kernel generator, which that step pins.
    out = {"diag": diag, "diag_names": np.array(DIAG), "forcing": F if per_step else F[-1:],
           "nsteps": np.int32(nsteps),
           "dels": np.float32(ts.dels), "seed": np.uint64(ts.seed), "doy0": np.int32(ts.doy0)}
    if mix is not None:
        out["diag_precision_mix"] = mix
    for k in STATE:
        out["state_" + k] = s[k]
    for k in TILE:
        out["tile_" + k] = np.asarray(getattr(ts, k))
    return out


def main():
    O.build()
    for name in CASES:
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **make_case(name))
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
