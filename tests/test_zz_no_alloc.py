"""cablegpu_cold_start_noalloc: the allocation-free cold start gives the
same state as cablegpu_cold_start, on two calls in a row into the same
context, and refuses contexts larger than its fixed staging array.

Kept in its own file, collected last, so it also runs after every other GPU
test in the same process (the staging array's address is resolved once per
device, on first use)."""
import numpy as np
import pytest

from cable_gb300 import workloads as W

pytestmark = pytest.mark.gpu

STATE = ["wb", "wbice", "tgg", "tggsn", "ssdn", "smass", "sdepth", "flags", "snowd", "ssdnn", "snage", "pudsto",
         "owetfac", "rtsoil", "tss", "cansto", "cplant", "csoil", "owb", "ebal_tot", "wbal_tot", "gammzz1"]


def _inputs(ts, k):
    # call 0: the workload's own cold start; call 1: a different one
    if k == 0:
        return ts.snowd0, ts.tgg0, ts.wb0
    return ts.snowd0[::-1].copy() * 0.5, np.clip(ts.tgg0 + 3.0, 250.0, 300.0), ts.wb0 * 0.9


def test_noalloc_cold_start_matches_cold_start_twice_in_a_row():
    from cable_gb300 import runtime as R
    ts = W.snow_grid(6000, seed=99, nsteps=4)
    ref = R.CableGPU(ts)
    na = R.CableGPU(ts)
    for ctx in (ref, na):
        ctx.set_synthetic_forcing(ts.seed, ts.doy0)
    for k in range(2):
        sn, tg, wb = _inputs(ts, k)
        ref.cold_start(sn, tg, wb)
        na.cold_start_noalloc(sn, tg, wb)
        for f in STATE:
            a, b = ref.get(f), na.get(f)
            np.testing.assert_allclose(b, a, rtol=0, atol=0, err_msg="call %d field %s" % (k, f))
        ref.run(1, 4)
        na.run(1, 4)
        ref.synchronize()
        na.synchronize()
        for f in ("out", "wb", "tgg", "snowd"):
            np.testing.assert_allclose(na.get(f), ref.get(f), rtol=1e-6, atol=1e-6, err_msg="call %d %s" % (k, f))
    ref.close()
    na.close()


def test_noalloc_cold_start_rejects_too_many_tiles():
    from cable_gb300 import runtime as R
    ts = W.grid(R.NOALLOC_MAX_TILES + 1, nsteps=1)
    g = R.CableGPU(ts)
    with pytest.raises(R.CableGPUError) as e:
        g.cold_start_noalloc(ts.snowd0, ts.tgg0, ts.wb0)
    assert e.value.code == -1 and "limit" in str(e.value)
    # the context stays usable through the allocating entry point
    g.cold_start(ts.snowd0, ts.tgg0, ts.wb0)
    g.set_synthetic_forcing(ts.seed)
    g.step(1)
    g.synchronize()
    g.close()
