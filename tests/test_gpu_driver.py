"""The drop-in boundary on the GPU: everything the offline driver reads from
the derived types between two cbm() calls (cable_serial.F90:594-740), with
the library's diagnostics on, checked step by step against the FP64 oracle
through the C ABI, and the per-tile parameter checks the Fortran shim runs
at set-up.

What the driver reads after cbm(): the runoff and snow melt it rescales by
dels (ssnow%smelt, rnof1, rnof2, runoff :602-605), the screen temperature of
its daily extremes (canopy%tscrn :607-608), the carbon fluxes of sumcflux
(:713; canopy%fgpp, fnpp, fpn, fra, frday, frp, frpw, frpr, frs), the inputs
of mass_balance / energy_balance (:725-728; cable_checks.F90:472-618; the
library runs both on the device: bal%ebal, wbal and their totals) and the
output writer's fluxes, temperatures, soil profiles and snow (:734-738)."""
import ctypes as C

import numpy as np
import pytest

import harness as H
import oracle_lib as O
from cable_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# driver-read fields with a tolerance: GPU diagnostics name (oracle name in
# harness.DIAG_MAP) and state fields
DRIVER_DIAG = ["fe_d", "fh_d", "fev", "fhv", "fhs", "fns", "fnv", "ga_d", "rnet_d", "fes", "fevc", "fevw",
               "tv_d", "trad_d", "tscrn", "qscrn", "fgpp_d", "frday_d", "fpn", "fnpp", "fnee", "frp", "frs", "frpw",
               "frpr", "runoff", "rnof1", "rnof2", "smelt", "delwc", "precis", "through"]
DRIVER_STATE = ["wb", "wbice", "tgg", "tggsn", "tss", "cansto"]


def test_driver_fields_every_step_against_the_oracle():
    from cable_gb300 import runtime as R
    ts = W.snow_grid(4000, seed=57, nsteps=24)
    n = 24
    F = O.forcing(ts, 0, n)
    g = R.from_tileset(ts, order=2)
    g.set_options(diag=True)
    st64, st32 = O.init_state(ts, 0), O.init_state(ts, 1)
    got = {k: [] for k in DRIVER_DIAG + DRIVER_STATE + ["cls"]}
    ref = {k: [] for k in got}
    mix = {k: [] for k in got}
    for k in range(n):
        g.set_forcing(F[k])
        g.step(k + 1, ts.dels)
        d64 = O.run(ts, st64, 1, ktau0=k + 1, forcing=F[k:k + 1], precision=0)
        d32 = O.run(ts, st32, 1, ktau0=k + 1, forcing=F[k:k + 1], precision=1)
        s64, s32 = O.split_state(st64), O.split_state(st32)
        for f in DRIVER_DIAG + ["cls"]:
            got[f].append(g.get(f)[0])
            ref[f].append(d64[H.DIAG_MAP[f]])
            mix[f].append(d32[H.DIAG_MAP[f]])
        for f in DRIVER_STATE:
            got[f].append(g.get(f))
            ref[f].append(s64[f][: got[f][-1].shape[0]].copy())
            mix[f].append(s32[f][: got[f][-1].shape[0]].copy())
    g.synchronize()
    g.close()
    bad = {}
    for f in DRIVER_DIAG + DRIVER_STATE:
        a, b, m = np.stack(got[f]), np.stack(ref[f]), np.stack(mix[f])
        rg, rm = H.compare(f, a, b), H.compare(f, m, b)
        assert "tol" in rg, f
        bad[f] = H.noise_criterion(rg, rm)
    assert not any(bad.values()), {k: v for k, v in bad.items() if v}
    # the snow flag of the soil evaporation agrees on all but the precision-noise tiles
    cls_g, cls_o = np.stack(got["cls"]), np.stack(ref["cls"])
    assert np.mean(np.abs(cls_g - cls_o) < 1e-6) > 0.999


def test_tile_parameters_are_checked_against_the_tables():
    """cablegpu_check_tile_param: the driver's per-tile parameters equal to
    the tables pass; one changed tile is refused with its tile number."""
    from cable_gb300 import runtime as R
    ts = W.grid(3000, nsteps=1)
    g = R.from_tileset(ts)
    for name in ("vcmax", "ejmax", "hc", "dleaf", "xfang", "a1gs", "g1"):
        tab = R.param_table(0, name)
        v = tab[ts.iveg - 1].astype(np.float32)
        g.check_tile_param(name, v)
        v[1234] *= 1.05
        with pytest.raises(R.CableGPUError) as e:
            g.check_tile_param(name, v)
        assert e.value.code == -1 and "tile 1235" in str(e.value), e.value
    for name in ("ssat", "sfc", "swilt", "bch", "hyds", "css"):
        tab = R.param_table(1, name)
        g.check_tile_param(name, tab[ts.isoilm - 1].astype(np.float32))
    fr = R.param_table(0, "froot").reshape(6, 17)
    g.check_tile_param("froot", fr[:, ts.iveg - 1].astype(np.float32))
    with pytest.raises(R.CableGPUError):
        g.check_tile_param("no_such_parameter", np.zeros(ts.mp, np.float32))
    g.close()


def test_per_tile_soil_albedo():
    """The per-tile bare-soil albedo (field "albsoil", soil%albsoil(:,1))
    defaults to the soil table: setting it to the table values changes
    nothing; a brighter soil raises the albedo of the bare tiles."""
    from cable_gb300 import runtime as R
    ts = W.grid(3000, nsteps=2)
    runs = []
    for mode in ("default", "table", "bright"):
        g = R.from_tileset(ts)
        g.set_options(diag=True)
        if mode != "default":
            alb = R.param_table(1, "albsoil_vis")[ts.isoilm - 1].astype(np.float32)
            if mode == "bright":
                alb = alb + 0.1
            g.set("albsoil", alb)
        g.step(1)
        g.step(2)
        runs.append({k: g.get(k) for k in ("out", "albedo_vis", "tgg")})
        g.close()
    for k in runs[0]:
        np.testing.assert_array_equal(runs[0][k], runs[1][k], err_msg=k)
    # barren and urban tiles off ice soil: a lake's soil albedo follows its
    # temperature (surface_albedosn) and an ice soil's is fixed
    bare = ((ts.iveg == 14) | (ts.iveg == 15)) & (ts.isoilm != 9)
    assert bare.sum() > 10
    assert np.all(runs[2]["albedo_vis"][0][bare] > runs[0]["albedo_vis"][0][bare])
    rest = (ts.iveg == 16) | (ts.isoilm == 9)
    np.testing.assert_array_equal(runs[2]["albedo_vis"][0][rest], runs[0]["albedo_vis"][0][rest])


def test_host_registered_buffers_step_like_any_host_buffers():
    """cablegpu_host_register page-locks the driver's own forcing and output
    arrays, and cablegpu_host_alloc provides page-locked memory for them
    (the Fortran shim's forc and outb): the pipelined host steps then
    give bitwise the outputs of ordinary buffers."""
    from cable_gb300 import runtime as R
    ts = W.grid(20000, seed=5, nsteps=4)
    cap = R.from_tileset(ts)
    cap.set_options(capture_forcing=True)
    forc = []
    for k in range(1, 4):
        cap.step(k)
        forc.append(np.ascontiguousarray(cap.get("forcing")))
    cap.close()
    outs = []
    for mode in ("plain", "register", "alloc"):
        g = R.from_tileset(ts)
        blk = None
        if mode == "alloc":
            blk = R.HostBlock([forc[0].shape, (8, ts.mp)])
            f, o = blk.arrays
            assert not f.any() and not o.any()   # zeroed
            assert f.ctypes.data % 256 == 0 and o.ctypes.data % 256 == 0
        else:
            f = np.zeros_like(forc[0])
            o = np.zeros((8, ts.mp), np.float32)
        if mode == "register":
            g.host_register(f)
            g.host_register(o)
        got = []
        for k in range(3):
            f[...] = forc[k]
            g.step_host(k + 1, f, o)
            g.synchronize()
            got.append(o.copy())
        if mode == "register":
            g.host_unregister(f)
            g.host_unregister(o)
        if blk is not None:
            ptr = blk.ptr
            blk.free()
            assert blk.L.cablegpu_host_free(C.c_void_p(ptr)) == -1   # released once only
        outs.append(got)
        g.close()
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            np.testing.assert_array_equal(a, b)


def test_batched_copy_back_equals_single_copies():
    """cablegpu_get_fields (one wait for many fields) gives the same arrays
    as cablegpu_get_field per field, for state of every storage type
    (double-FP32, FP64, FP32, bytes) and diagnostics."""
    from cable_gb300 import runtime as R
    ts = W.snow_grid(6000, seed=9, nsteps=3)
    g = R.from_tileset(ts)
    g.set_options(diag=True)
    for k in (1, 2, 3):
        g.step(k)
    names = ["wb", "wbice", "gammzz1", "tgg", "tggsn", "flags", "snowd", "cansto", "out", "fev", "runoff", "tscrn",
             "ebal_tot", "wbal_tot"]
    many = g.get_many(names)
    for n in names:
        np.testing.assert_array_equal(many[n], g.get(n), err_msg=n)
    # an unknown field id is refused
    rc = g.L.cablegpu_get_fields(g.h, 1, (R.C.c_int * 1)(-1), (R.C.c_void_p * 1)(None))
    assert rc == -1, rc
    g.close()


def test_tune_blocks_leaves_the_run_unchanged():
    """cablegpu_tune_blocks times block sizes on the context's own state and
    puts the state back: the steps after it are bitwise those of a context
    that was not tuned (results do not depend on block sizes either)."""
    from cable_gb300 import runtime as R
    ts = W.snow_grid(20000, seed=13, nsteps=12)
    runs = []
    for tune in (False, True):
        g = R.from_tileset(ts)
        g.run(1, 4)
        g.synchronize()
        if tune:
            blocks, ms = g.tune_blocks(5, 2)
            assert len(blocks) == 5 and all(b in (32, 64, 128, 256) for b in blocks) and ms > 0
        g.run(5, 8)
        g.synchronize()
        runs.append({k: g.get(k) for k in ("out", "wb", "tgg", "snowd", "cansto", "wbal_tot", "tile_status")})
        g.close()
    for k in runs[0]:
        np.testing.assert_array_equal(runs[0][k], runs[1][k], err_msg=k)
