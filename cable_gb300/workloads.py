"""Seeded synthetic tile sets for the CABLE cbm() timestep.

The reference drives cbm() from netCDF site / gridded files (the site forcing
``TumbaFluxnet.1.3_met.nc`` and ``gridinfo_CSIRO_1x1.nc`` are not available);
these generators stand in for them with the distributions the benchmark
workloads specify.  Per-step met forcing is not generated here: it is produced
inside the timestep kernel from (seed, tile, step) with a counter-based RNG, so
only the per-tile static inputs below live in memory.

Every workload returns a :class:`TileSet` of numpy arrays, one entry per tile.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

__all__ = ["TileSet", "site5", "grid", "snow_grid", "WORKLOADS", "make"]

TFRZ = 273.16


@dataclass
class TileSet:
    """Static inputs for ``mp`` tiles (all arrays have length ``mp``)."""

    name: str
    iveg: np.ndarray          # int32, PFT 1..17
    isoilm: np.ndarray        # int32, soil type 1..9
    vlai: np.ndarray          # float64, LAI before snow burial
    lat: np.ndarray           # float32, degrees north
    lonphase: np.ndarray      # float32, local-time offset (hours, [0, 24))
    tbase: np.ndarray         # float32, base air temperature of the forcing (K)
    swscale: np.ndarray       # float32, shortwave scale factor
    snowd0: np.ndarray        # float64, initial snow water equivalent (kg/m2)
    tgg0: np.ndarray          # float64, initial soil temperature (K), all layers
    wb0: np.ndarray           # float64, initial volumetric soil moisture, all layers
    seed: int = 12345
    doy0: int = 1
    dels: float = 1800.0
    nsteps: int = 48
    extra: dict = field(default_factory=dict)

    @property
    def mp(self) -> int:
        return int(self.iveg.shape[0])

    def subset(self, idx) -> "TileSet":
        """Tiles ``idx`` as a new set (forcing is keyed on the new tile index)."""
        if not isinstance(idx, slice):
            idx = np.asarray(idx)
        g = lambda a: np.ascontiguousarray(a[idx])
        return TileSet(self.name + "[sub]", g(self.iveg), g(self.isoilm), g(self.vlai), g(self.lat),
                       g(self.lonphase), g(self.tbase), g(self.swscale), g(self.snowd0), g(self.tgg0),
                       g(self.wb0), self.seed, self.doy0, self.dels, self.nsteps, dict(self.extra))


def _lognormal_lai(rng, n):
    # LAI lognormal (median 2, sigma 0.8) clipped to [0.1, 8]
    return np.clip(np.exp(np.log(2.0) + 0.8 * rng.standard_normal(n)), 0.1, 8.0)


def site5(seed: int = 12345, nsteps: int = 17520) -> TileSet:
    """One site, five tiles (PFT 1, 2, 5, 6, 9) on soil type 2, no jitter.

    Latitude is Tumbarumba's (-35.66); LAI per PFT is a stated choice
    (4.0, 5.0, 1.5, 2.0, 3.0) since the gridded LAI file is not available.
    """
    iveg = np.array([1, 2, 5, 6, 9], np.int32)
    n = iveg.size
    return TileSet("site5", iveg, np.full(n, 2, np.int32), np.array([4.0, 5.0, 1.5, 2.0, 3.0]),
                   np.full(n, -35.66, np.float32), np.zeros(n, np.float32), np.full(n, 288.0, np.float32),
                   np.ones(n, np.float32), np.zeros(n), np.full(n, 285.0), np.full(n, 0.25),
                   seed=seed, nsteps=nsteps)


def grid(mp: int = 1_000_000, seed: int = 12345, nsteps: int = 48) -> TileSet:
    """Gridded tiles: PFT uniform 1..17, soil 1..9, LAI lognormal, per-tile
    temperature offset N(0, 10 K), SW scale U(0.5, 1.2), latitude U(-60, 70),
    local-time phase U(0, 24 h); soil at 0.25 m3/m3 and 285 K, no snow."""
    rng = np.random.default_rng(seed)
    iveg = rng.integers(1, 18, mp).astype(np.int32)
    isoilm = rng.integers(1, 10, mp).astype(np.int32)
    vlai = _lognormal_lai(rng, mp)
    lat = rng.uniform(-60.0, 70.0, mp).astype(np.float32)
    lonphase = rng.uniform(0.0, 24.0, mp).astype(np.float32)
    tbase = (288.0 + 10.0 * rng.standard_normal(mp)).astype(np.float32)
    swscale = rng.uniform(0.5, 1.2, mp).astype(np.float32)
    return TileSet("grid", iveg, isoilm, vlai, lat, np.minimum(lonphase, np.float32(23.999)), tbase, swscale,
                   np.zeros(mp), np.full(mp, 285.0), np.full(mp, 0.25), seed=seed, nsteps=nsteps)


def snow_grid(mp: int = 4_000_000, seed: int = 12345, nsteps: int = 480, snow_frac: float = 0.4,
              snow_depth_mean: float = 0.3) -> TileSet:
    """Uneven gridded tiles: as :func:`grid` but with a base air temperature
    U(250, 300 K) and ``snow_frac`` of the tiles snow-covered with depth
    Exp(mean ``snow_depth_mean`` m) at the cold-start density 120 kg/m3, which
    gives no snow, thin single-layer snow and 3-layer packs.  Initial soil
    temperature follows the air (clamped to [255, 285] K)."""
    ts = grid(mp, seed, nsteps)
    rng = np.random.default_rng(seed + 1)
    ts.tbase = rng.uniform(250.0, 300.0, mp).astype(np.float32)
    snowy = rng.random(mp) < snow_frac
    depth = rng.exponential(snow_depth_mean, mp)
    ts.snowd0 = np.where(snowy, depth * 120.0, 0.0)
    ts.tgg0 = np.clip(ts.tbase.astype(np.float64) + 5.0, 255.0, 285.0)
    ts.name = "snow_grid"
    return ts


WORKLOADS = {
    "site5": site5,
    "grid": grid,
    "snow_grid": snow_grid,
}


def make(name: str, **kw) -> TileSet:
    return WORKLOADS[name](**kw)
