"""The largest context (CABLEGPU_MAX_TILES tiles, ~34 GB of device arena):
its kernels address the highest rows of the multi-row fields (diagnostics
row 62, radiation record row 51) at the last tiles, where 32-bit row offsets
come closest to 2^31.  Every tile i is given the description and the forcing
of tile i mod 1024 of a 1024-tile context, so its outputs, state and
diagnostics must equal that context's bit for bit (each tile's arithmetic
depends on its own inputs only)."""
import numpy as np
import pytest

from cable_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NSMALL = 1024
STEPS = 2
COMPARE = ["out", "tgg", "wb", "snowd"]


@pytest.fixture(scope="module")
def runtime():
    from cable_gb300 import runtime as R
    R.load()
    return R


def test_largest_context_equals_its_repeated_small_context(runtime):
    R = runtime
    names = [n for n, v in R.fields().items() if v[3] == R.KIND_DIAG]
    diag_rows = [names[0], names[-1]]
    small = W.snow_grid(NSMALL, nsteps=STEPS)
    g = R.from_tileset(small, order=1)
    g.set_options(diag=True, capture_forcing=True)
    forcing = []
    for n in range(STEPS):
        g.step(1 + n)
        forcing.append(g.get("forcing"))
    ref = {k: g.get(k) for k in COMPARE + diag_rows}
    g.close()

    n = R.MAX_TILES
    rep = np.arange(n) % NSMALL
    big = R.from_tileset(small.subset(rep), order=1)
    big.set_options(diag=True)
    for s in range(STEPS):
        big.set_forcing(np.ascontiguousarray(forcing[s][:, rep]))
        big.step(1 + s)
    big.synchronize()
    for k in COMPARE + diag_rows:
        got = big.get(k)
        want = ref[k][..., rep]
        assert got.shape == want.shape, k
        assert np.array_equal(got, want), k
    big.close()
