"""GPU timestep against the FP64 CPU oracle on identical forcing.

Tolerances (the benchmark spec): fluxes 1e-3 relative with a 1 W/m2 floor
(carbon fluxes: a 1e-7 g C/m2/s floor), temperatures 0.01 K, soil moisture
1e-5 m3/m3.  A few tiles per thousand can flip a branch of the iterative
canopy solution or of the snow layering in FP32 (as the reference's own FP32
build does against FP64), so on gridded workloads the check
(harness.noise_criterion) counts the values out of tolerance against the
count of the reference's REAL=FP32 / r_2=FP64 build on the same inputs, and
holds the RMS error of the unflipped values to the tolerance."""
import numpy as np
import pytest

import harness as H
from cable_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# the outputs the accuracy targets name (latent and sensible heat, GPP,
# canopy and soil temperature, soil moisture) and the fluxes that make them up
FIELDS = ["fe_d", "fh_d", "ga_d", "rnet_d", "fes", "fevc", "tv_d", "trad_d", "tgg", "tggsn", "wb", "wbice",
          "fgpp_d", "fpn", "frday_d"]


@pytest.fixture(scope="module")
def runtime():
    from cable_gb300 import runtime as R
    R.load()
    return R


def test_site5_every_tile_within_tolerance(runtime):
    ts = W.site5(nsteps=96)
    gs, gd, os_, od, _ = H.run_pair(ts, 96)
    rep = H.parity_report(gs, gd, os_, od)
    for k in FIELDS:
        assert rep[k]["frac_within"] == 1.0, (k, rep[k])
    assert np.abs(gd["ebal"]).max() < 0.01
    assert np.abs(gd["drybal"]).max() < 0.01
    assert np.array_equal(gd["dryleaf_passes"], od["dryleaf_passes"])


@pytest.mark.parametrize("name", ["grid", "snow_grid"])
def test_gridded_parity_matches_reference_precision_noise(oracle, runtime, name):
    ts = W.make(name, mp=20000, nsteps=48)
    gs, gd, os_, od, F = H.run_pair(ts, 48)
    rep = H.parity_report(gs, gd, os_, od)
    # the reference's own precision mix on the same forcing
    st32 = oracle.init_state(ts, 1)
    od32 = oracle.run(ts, st32, 48, forcing=F, precision=1)
    os32 = oracle.split_state(st32)
    gs32 = {k: os32[k] for k in H.STATE_FIELDS}
    gd32 = {gk: od32[ok] for gk, ok in H.DIAG_MAP.items()}
    ref = H.parity_report(gs32, gd32, os_, od)
    bad = {k: H.noise_criterion(rep[k], ref[k]) for k in FIELDS}
    assert not any(bad.values()), {k: (v, rep[k], ref[k]) for k, v in bad.items() if v}
    if name == "grid":
        # no snow: the RMS itself is inside the tolerance; with snow a few
        # tiles flip snow layering and dominate the RMS exactly as they do
        # for the reference's own FP32 build (checked above)
        for k in ("fe_d", "fh_d", "tv_d", "tgg"):
            assert rep[k]["rms"] < rep[k]["tol"], (k, rep[k])
    assert np.abs(gd["ebal"]).max() < 0.05
    assert np.array_equal(gs["flags"][0] & 1, os_["isflag"][0].astype(np.int32)) or \
        np.mean((gs["flags"][0] & 1) == os_["isflag"][0]) > 0.999


def test_plain_kernels_equal_the_diagnostics_kernels(runtime):
    """The benchmarked instantiations (diagnostics off) compute bitwise the
    outputs and state of the diagnostics instantiations that the per-step
    flux comparisons run: every output row every step, and the state after
    24 steps, stepped directly and replayed as CUDA graphs."""
    R = runtime
    ts = W.snow_grid(20000, nsteps=24)
    names = [n for n, v in R.fields().items() if v[3] == R.KIND_STATE] + ["tile_status"]
    runs = []
    for diag in (False, True):
        g = R.from_tileset(ts, order=2)
        g.set_options(diag=diag)
        outs = []
        for n in range(24):
            g.step(1 + n, ts.dels)
            outs.append(g.get("out"))
        runs.append((outs, {k: g.get(k) for k in names}))
        g.close()
    g = R.from_tileset(ts, order=2)
    g.run(1, 24, ts.dels)
    g.synchronize()
    graph = {k: g.get(k) for k in names}
    g.close()
    (o0, s0), (o1, s1) = runs
    for n in range(24):
        np.testing.assert_array_equal(o0[n], o1[n], err_msg="out, step %d" % (n + 1))
    for k in names:
        if k == "tile_status":   # the dryLeaf bits are recorded by the diagnostics kernel only
            np.testing.assert_array_equal(s0[k] & ~(R.TILE_DRYLEAF_NOCONV | R.TILE_EVAPFBL),
                                          s1[k] & ~(R.TILE_DRYLEAF_NOCONV | R.TILE_EVAPFBL), err_msg=k)
            continue
        np.testing.assert_array_equal(s0[k], s1[k], err_msg=k)
        np.testing.assert_array_equal(s0[k], graph[k], err_msg="graph " + k)


@pytest.mark.parametrize("blocks", [[128, 128, 128, 128, 128], [256, 64, 64, 64, 64], [64, 32, 32, 32, 32]])
def test_canopy_pool_equals_per_lane_schedule(runtime, blocks):
    """The canopy kernel's dryLeaf passes run as a block pool (default) or
    per lane: outputs every step and state after 24 steps bitwise equal, with
    diagnostics off and on (20,003 tiles: the last block has threads beyond
    the last tile, which take part in the pool's barriers as ghosts)."""
    R = runtime
    ts = W.snow_grid(20003, nsteps=24)
    names = [n for n, v in R.fields().items() if v[3] == R.KIND_STATE]
    for diag in (False, True):
        runs = []
        for sched in ("lanes", "pool"):
            g = R.from_tileset(ts, order=2)
            g.set_blocks(blocks)
            g.set_options(diag=diag)
            g.set_canopy_schedule(sched)
            outs = []
            for n in range(24):
                g.step(1 + n, ts.dels)
                outs.append(g.get("out"))
            st = {k: g.get(k) for k in names}
            if diag:
                st["dryleaf_passes"] = g.get("dryleaf_passes")
            runs.append((outs, st))
            g.close()
        (o0, s0), (o1, s1) = runs
        for n in range(24):
            np.testing.assert_array_equal(o0[n], o1[n], err_msg="diag %d out, step %d" % (diag, n + 1))
        for k in s0:
            np.testing.assert_array_equal(s0[k], s1[k], err_msg="diag %d %s" % (diag, k))


def test_host_forcing_path_matches_synthetic(runtime):
    """The drop-in path (forcing uploaded from the host every step) gives the
    same state as the in-kernel generator when fed its forcing."""
    R = runtime
    ts = W.snow_grid(3000, nsteps=6)
    g = R.from_tileset(ts)
    g.set_options(capture_forcing=True)
    F = []
    for n in range(6):
        g.step(1 + n)
        F.append(g.get("forcing"))
    a = {k: g.get(k) for k in ("wb", "tgg", "out", "snowd")}
    g.close()
    h = R.from_tileset(ts)
    for n in range(6):
        h.set_forcing(F[n])
        h.step(1 + n)
    b = {k: h.get(k) for k in ("wb", "tgg", "out", "snowd")}
    h.close()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_graph_replay_equals_single_steps_and_tile_order_is_irrelevant(runtime):
    R = runtime
    ts = W.snow_grid(5000, nsteps=20)
    runs = []
    for order, graph in ((0, True), (0, False), (1, True)):
        g = R.from_tileset(ts, order=order)
        if graph:
            g.run(1, 20)
        else:
            for n in range(20):
                g.step(1 + n)
        g.synchronize()
        runs.append({k: g.get(k) for k in ("wb", "wbice", "tgg", "tggsn", "out", "snowd", "cplant")})
        # 5 kernels per step; graph replay (16 of the 20 steps) adds the
        # step-counter kernel of each replayed step
        assert g.launch_count() == 100 + (16 if graph else 0)
        g.close()
    for r in runs[1:]:
        for k in r:
            assert np.array_equal(runs[0][k], r[k]), k


def test_gpu_forcing_generator_matches_cpu(oracle, runtime):
    R = runtime
    ts = W.grid(4000, nsteps=3)
    g = R.from_tileset(ts)
    g.set_options(capture_forcing=True)
    for n in range(3):
        g.step(1 + n)
    fg = g.get("forcing")
    g.close()
    fc = oracle.forcing(ts, 2, 1)[0]
    for i, name in enumerate(oracle.FORCING_FIELDS):
        np.testing.assert_allclose(fg[i], fc[i], rtol=2e-5, atol=2e-5 * max(1.0, float(np.abs(fc[i]).max())), err_msg=name)
    assert np.array_equal(fg[3] > 0, fc[3] > 0)      # precipitation events identical


def test_field_roundtrip_and_restart(runtime):
    """get/set are exact inverses; a state saved at step 6 and restored into a
    fresh context continues like the uninterrupted run.  Soil water and ice
    are carried on the device with a 48-bit significand spread over two FP32
    words whose low word can reach far below the FP64 grid, so a restart
    through the FP64 interface (like the reference's r_2 restart file) rounds
    them at ~1e-16 and the continuation agrees to roundoff, not bitwise."""
    R = runtime
    ts = W.snow_grid(3000, nsteps=12)
    g = R.from_tileset(ts)
    g.run(1, 6)
    state_names = [n for n, v in g.fields.items() if v[3] == R.KIND_STATE]
    saved = {n: g.get(n) for n in state_names}
    g.run(7, 6)
    ref = {k: g.get(k) for k in ("wb", "tgg", "out")}
    g.close()
    h = R.from_tileset(ts)
    for n, v in saved.items():
        h.set(n, v)
        assert np.array_equal(h.get(n), v), n
    h.run(7, 6)
    np.testing.assert_allclose(h.get("wb"), ref["wb"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(h.get("tgg"), ref["tgg"], rtol=0, atol=1e-4)
    np.testing.assert_allclose(h.get("out"), ref["out"], rtol=1e-4, atol=1e-3)
    h.close()


def test_nonfinite_input_is_reported_not_trapped(runtime):
    """Host-side fault injection: a NaN in the forcing must surface as
    CABLEGPU_ERR_NONFINITE at the next synchronisation, and the context stays
    usable."""
    R = runtime
    ts = W.grid(1000, nsteps=2)
    g = R.from_tileset(ts)
    g.set_options(capture_forcing=True)
    g.step(1)
    f = g.get("forcing")
    f[5, 17] = np.nan          # air temperature of one tile
    g.set_forcing(f)
    g.step(2)
    with pytest.raises(R.CableGPUError) as e:
        g.synchronize()
    assert e.value.code == -3
    st = g.get("tile_status")[0]
    assert st[17] & R.TILE_NONFINITE and st[17] & R.TILE_FORCING_RANGE
    assert not np.any(np.delete(st, 17) & (R.TILE_NONFINITE | R.TILE_FORCING_RANGE))
    g.set_synthetic_forcing(ts.seed)
    ok = R.from_tileset(ts)
    ok.step(1)
    ok.synchronize()
    ok.close()
    g.close()


def test_diagnostics_disabled_is_an_error(runtime):
    R = runtime
    ts = W.grid(256, nsteps=1)
    g = R.from_tileset(ts)
    g.step(1)
    with pytest.raises(R.CableGPUError) as e:
        g.get("fev")
    assert e.value.code == -4
    g.close()


def test_medlyn_switch_matches_oracle(oracle, runtime):
    ts = W.grid(4000, nsteps=12)
    gs, gd, os_, od, F = H.run_pair(ts, 12, medlyn=True)
    rep = H.parity_report(gs, gd, os_, od)
    st32 = oracle.init_state(ts, 1)
    od32 = oracle.run(ts, st32, 12, forcing=F, precision=1, medlyn=True)
    os32 = oracle.split_state(st32)
    ref = H.parity_report({k: os32[k] for k in H.STATE_FIELDS}, {gk: od32[ok] for gk, ok in H.DIAG_MAP.items()},
                          os_, od)
    bad = {k: H.noise_criterion(rep[k], ref[k]) for k in ("fe_d", "fh_d", "tv_d", "tgg", "wb", "fgpp_d", "frday_d")}
    assert not any(bad.values()), {k: (v, rep[k], ref[k]) for k, v in bad.items() if v}


def test_autotuned_order_and_block_sizes_leave_results_unchanged(runtime):
    """Tile order and block sizes (chosen by the autotuner, or set by hand)
    change only the speed: every field is bitwise the same."""
    R = runtime
    ts = W.snow_grid(20000, nsteps=6)
    fields = ("wb", "wbice", "tgg", "tggsn", "out", "snowd", "cplant", "rtsoil")
    runs = []
    for order, blocks in ((0, None), (-1, None), (2, [64, 256, 32, 96, 128]), (1, [256, 64, 128, 32, 256]), (3, None)):
        g = R.from_tileset(ts, order=order)
        o, b = g.config()
        assert o in (0, 1, 2, 3) and all(x % 32 == 0 and 32 <= x <= 256 for x in b)
        if blocks:
            g.set_blocks(blocks)
            assert g.config()[1] == blocks
        g.run(1, 6)
        g.synchronize()
        runs.append({k: g.get(k) for k in fields})
        g.close()
    for r in runs[1:]:
        for k in fields:
            assert np.array_equal(runs[0][k], r[k]), k
    with pytest.raises(R.CableGPUError):
        g = R.from_tileset(ts)
        try:
            g.set_blocks([100, 128, 128, 128, 128])
        finally:
            g.close()


def test_pipelined_host_io_step_equals_set_forcing_step_get(runtime):
    """cablegpu_step_host (copies overlapped with neighbouring steps) gives
    bitwise the outputs and state of set_forcing + step + get_field."""
    R = runtime
    ts = W.snow_grid(30000, nsteps=5)
    g = R.from_tileset(ts)
    g.set_options(capture_forcing=True)
    F = []
    for n in range(5):
        g.step(1 + n)
        F.append(g.get("forcing"))
    g.close()
    a = R.from_tileset(ts)
    outs_a = []
    for n in range(5):
        a.set_forcing(F[n])
        a.step(1 + n)
        outs_a.append(a.get("out"))
    b = R.from_tileset(ts, order=2)
    outs_b = [np.empty((8, ts.mp), np.float32) for _ in range(5)]
    for n in range(5):
        b.step_host(1 + n, np.ascontiguousarray(F[n]), outs_b[n])
    b.synchronize()
    for n in range(5):
        assert np.array_equal(outs_a[n], outs_b[n]), n
    for k in ("wb", "tgg", "snowd", "cansto"):
        assert np.array_equal(a.get(k), b.get(k)), k
    a.close()
    b.close()


@pytest.mark.parametrize("solve", ["fp64", "fp32_change"])
def test_site5_full_year_against_oracle(oracle, runtime, solve):
    """The benchmark's site configuration over a full year (5 tiles, PFTs
    1, 2, 5, 6, 9, soil type 2, 17,520 half-hour steps, replayed as CUDA
    graphs) against the FP64 oracle on the same synthetic forcing, with the
    FP64 soil solves (the default) and with the FP32 change-form option: no
    drift in soil temperature or moisture from either solve or from the
    double-FP32 soil water, and the cumulative energy and water balance
    residuals stay as closed as the oracle's."""
    R = runtime
    ts = W.site5(nsteps=17520)
    g = R.from_tileset(ts)
    g.set_soil_solve(solve)
    g.run(1, 17520)
    g.synchronize()
    gs = {k: g.get(k) for k in ("wb", "wbice", "tgg", "snowd", "ebal_tot", "wbal_tot", "cansto", "csoil", "cplant")}
    g.close()
    st = oracle.init_state(ts, 0)
    oracle.run(ts, st, 17520, precision=0)
    os_ = oracle.split_state(st)
    # measured over the year (FP32 change form): tgg 0.005 K, wb 8e-7,
    # ebal_tot 1.5, wbal_tot 8e-5, csoil 0.14 (of 623) -- the same size as
    # the REAL=FP32 oracle's own drift
    print("site5 year, %s solves: tgg %.3g K, wb %.3g, ebal_tot %.3g, wbal_tot %.3g, csoil %.3g" % (
        solve, np.abs(gs["tgg"] - os_["tgg"]).max(), np.abs(gs["wb"] - os_["wb"]).max(),
        np.abs(gs["ebal_tot"] - os_["ebal_tot"]).max(), np.abs(gs["wbal_tot"] - os_["wbal_tot"]).max(),
        np.abs(gs["csoil"] - os_["csoil"]).max()))
    assert np.abs(gs["tgg"] - os_["tgg"]).max() < 0.02                  # K after a year
    assert np.abs(gs["wb"] - os_["wb"]).max() < 1e-5                    # m3/m3 after a year
    assert np.abs(gs["wbice"] - os_["wbice"]).max() < 1e-5
    assert np.abs(gs["cansto"] - os_["cansto"]).max() < 1e-4            # mm
    # cumulative balance residuals (W/m2 and mm summed over the year)
    assert np.abs(gs["ebal_tot"] - os_["ebal_tot"]).max() < 5.0
    assert np.abs(gs["wbal_tot"] - os_["wbal_tot"]).max() < 1e-3
    np.testing.assert_allclose(gs["csoil"], os_["csoil"], rtol=1e-3, atol=0.5)   # g C/m2
    np.testing.assert_allclose(gs["cplant"], os_["cplant"], rtol=1e-3, atol=0.5)


@pytest.mark.parametrize("solve", ["fp64", "fp32_change"])
def test_snow_grid_full_year_against_oracle(oracle, runtime, solve):
    """256 snow_grid tiles (40 % snow-covered at the start, air 250-300 K)
    over a year, against the FP64 oracle.  Snow layering and melt are
    threshold events: two FP32 builds of the reference algorithm (the
    REAL=FP32 / r_2=FP64 mix compiled with and without FMA contraction)
    each flip a different 2-4 tiles by tens of kg/m2 of snow over the
    year, and 0-2 tiles by more than 0.1 K of soil temperature, so snow
    depth is checked as the fraction of tiles within 1 kg/m2 and soil
    temperature as a count of flipped tiles plus the RMS of the others.  The
    water balance stays as closed as the FP64 oracle's (with the FP32
    change-form option, thanks to its flux-form soil water update) and soil
    moisture and temperature do not drift; both soil solves."""
    R = runtime
    ts = W.snow_grid(mp=256, nsteps=17520)
    g = R.from_tileset(ts)
    g.set_soil_solve(solve)
    g.run(1, 17520)
    g.synchronize()
    gs = {k: np.asarray(g.get(k), np.float64) for k in ("wb", "tgg", "snowd", "wbal_tot", "csoil", "cplant")}
    g.close()
    st = oracle.init_state(ts, 0)
    oracle.run(ts, st, 17520, precision=0)
    o = {k: np.asarray(v, np.float64).reshape(gs[k].shape) for k, v in oracle.split_state(st).items() if k in gs}
    rms = lambda k: float(np.sqrt(np.mean((gs[k] - o[k]) ** 2)))
    # measured: wbal_tot rms 0.011 mm (the REAL=FP32 oracle: 0.011), wb rms
    # 2.2e-4, snow depth within 1 kg/m2 on 252 of 256 tiles; soil
    # temperature: 0-2 tiles flipped beyond 0.1 K (the FP32 oracle builds:
    # 0-2), the rest within 0.01 K RMS
    dt0 = np.abs(gs["tgg"] - o["tgg"])
    print("snow_grid year, %s solves: wbal_tot rms %.3g mm, wb rms %.3g, tgg flipped %d, snowd within 1 kg/m2 %.4f" % (
        solve, rms("wbal_tot"), rms("wb"), int((dt0.max(axis=0) > 0.1).sum()),
        float(np.mean(np.abs(gs["snowd"] - o["snowd"]) <= 1.0))))
    assert rms("wbal_tot") < 0.05                                       # mm over the year
    assert rms("wb") < 5e-4                                             # m3/m3
    dt = np.abs(gs["tgg"] - o["tgg"])
    flipped = dt.max(axis=0) > 0.1                                      # K, per tile
    assert flipped.sum() <= 4, np.where(flipped)[0]
    assert np.sqrt(np.mean(dt[:, ~flipped] ** 2)) < 0.02                # K
    assert np.mean(np.abs(gs["snowd"] - o["snowd"]) <= 1.0) >= 0.95     # kg/m2
    for k in ("csoil", "cplant"):
        assert np.mean(np.abs(gs[k] - o[k]) <= np.maximum(1e-3 * np.abs(o[k]), 0.5)) >= 0.95, k


SWITCH_SETS = {
    "soil_thermal_fix": dict(soil_thermal_fix=True),
    "litter": dict(litter=True),
    "l_rev_corr": dict(l_rev_corr=True),
    "fwsoil_nonlinear": dict(fwsoil_switch="non-linear extrapolation"),
    "fwsoil_lai_ktaul": dict(fwsoil_switch="Lai and Ktaul 2000"),
    "potev_pm": dict(ssnow_potev="P-M"),
    "reduce_soilevp": dict(l_new_reduce_soilevp=True),
    "runoff_speed": dict(l_new_runoff_speed=True),
    "soil_resp_off": dict(diag_soil_resp="OFF"),
    "all": dict(medlyn=True, soil_thermal_fix=True, litter=True, l_rev_corr=True,
                fwsoil_switch="non-linear extrapolation", ssnow_potev="P-M", l_new_reduce_soilevp=True,
                l_new_runoff_speed=True, diag_soil_resp="OFF"),
}
# the field each switch must move on the GPU, and by how much
SWITCH_LIVE = {"soil_thermal_fix": ("tgg", 0.05), "litter": ("fhs", 0.5), "l_rev_corr": ("tgg", 0.01),
               "fwsoil_nonlinear": ("fevc", 1.0), "fwsoil_lai_ktaul": ("fevc", 1.0), "potev_pm": ("fes", 1.0),
               "reduce_soilevp": ("fes", 1.0), "runoff_speed": ("wb", 1e-4), "soil_resp_off": ("frs", 1e-8),
               "all": ("tgg", 0.05)}


@pytest.mark.parametrize("which", list(SWITCH_SETS))
def test_science_switches_match_oracle(oracle, runtime, which):
    """The alternative science switches (soil_thermal_fix: conductivity and
    soil heat parameters; litter: litter resistances in define_canopy;
    l_rev_corr: revised soil-coupling derivatives; and all of them with
    medlyn) on snowy, freezing tiles against the FP64 oracle with the same
    switches, with the default configuration's criterion: RMS and fraction
    of tiles within tolerance against the reference's own FP32 build with
    the same switches.  Each switch is live on the GPU (results move)."""
    sw = SWITCH_SETS[which]
    ts = W.snow_grid(8000, nsteps=24)
    gs, gd, os_, od, F = H.run_pair(ts, 24, **sw)
    rep = H.parity_report(gs, gd, os_, od)
    st32 = oracle.init_state(ts, 1)
    od32 = oracle.run(ts, st32, 24, forcing=F, precision=1, **sw)
    os32 = oracle.split_state(st32)
    ref = H.parity_report({k: os32[k] for k in H.STATE_FIELDS}, {gk: od32[ok] for gk, ok in H.DIAG_MAP.items()},
                          os_, od)
    bad = {k: H.noise_criterion(rep[k], ref[k])
           for k in ("tgg", "tggsn", "wb", "wbice", "ga_d", "fe_d", "fh_d", "tv_d", "fes", "fgpp_d", "frday_d")}
    assert not any(bad.values()), {k: (v, rep[k], ref[k]) for k, v in bad.items() if v}
    assert np.abs(gd["ebal"]).max() < 0.05
    # soil respiration (frs) and transpiration (fevc) against the oracle too
    rms = lambda e: float(np.sqrt(np.mean(e ** 2)))
    for k in ("frs", "fevc"):
        ref = np.asarray(od[H.DIAG_MAP[k]], np.float64)
        err = np.abs(np.asarray(gd[k], np.float64) - ref)
        err32 = np.abs(np.asarray(od32[H.DIAG_MAP[k]], np.float64) - ref)
        assert rms(err) <= max(3 * rms(err32), 1e-3 * np.abs(ref).max() + 1e-12), (k, rms(err), rms(err32))
    g0, d0, _, _, _ = H.run_pair(ts, 24)
    field, thr = SWITCH_LIVE[which]
    a0 = np.asarray(g0[field] if field in g0 else d0[field], np.float64)
    a1 = np.asarray(gs[field] if field in gs else gd[field], np.float64)
    assert np.abs(a1 - a0).max() > thr, (which, field, np.abs(a1 - a0).max())


def test_tile_status_matches_the_oracle_and_flags_bad_forcing(oracle, runtime):
    """The per-tile status bits: dryLeaf non-convergence and the reference's
    'oldevapfbl not right' condition agree with the oracle step by step
    (up to the precision-noise tiles), the seeded forcing is inside the
    driver's check ranges, and finite out-of-range forcing on two tiles sets
    their forcing bit only.  (The two dryLeaf bits are recorded with
    diagnostics on.)"""
    R = runtime
    ts = W.snow_grid(20000, nsteps=12)
    n = 12
    F = oracle.forcing(ts, 0, n)
    g = R.from_tileset(ts)
    g.set_options(diag=True)
    st = oracle.init_state(ts, 0)
    agree_nc, agree_ev, any_nc = [], [], 0
    for k in range(n):
        g.set("tile_status", 0)
        g.set_forcing(F[k])
        g.step(k + 1, ts.dels)
        bits = g.get("tile_status")[0]
        d = oracle.run(ts, st, 1, ktau0=k + 1, forcing=F[k:k + 1], precision=0)
        assert not np.any(bits & (R.TILE_FORCING_RANGE | R.TILE_NONFINITE))
        nc_o = np.asarray(d["dryleaf_noconv"]) > 0
        ev_o = np.asarray(d["evapfbl_err"]) > 0
        agree_nc.append(np.mean((bits & R.TILE_DRYLEAF_NOCONV > 0) == nc_o))
        agree_ev.append(np.mean((bits & R.TILE_EVAPFBL > 0) == ev_o))
        any_nc += int(nc_o.sum())
    assert min(agree_nc) > 0.998 and min(agree_ev) > 0.998, (agree_nc, agree_ev)
    # finite but out-of-range forcing: tile 17 at 340 K, tile 23 with 80 m/s wind
    f = F[0].copy()
    f[5, 17] = 340.0
    f[7, 23] = 80.0
    g.set("tile_status", 0)
    g.set_forcing(f)
    g.step(n + 1, ts.dels)
    g.synchronize()
    bits = g.get("tile_status")[0]
    assert bits[17] & R.TILE_FORCING_RANGE and bits[23] & R.TILE_FORCING_RANGE
    assert not np.any(np.delete(bits, [17, 23]) & R.TILE_FORCING_RANGE)
    g.close()


def test_host_layout_in_device_order_matches_caller_order(oracle, runtime):
    """cablegpu_set_host_layout(1): host forcing and outputs in the device
    tile order (cablegpu_tile_order) give bitwise the same steps as the
    caller-order buffers."""
    R = runtime
    ts = W.snow_grid(5000, nsteps=6)
    n, mp = 6, ts.mp
    F = oracle.forcing(ts, 0, n)
    runs = []
    for layout in (0, 1):
        g = R.from_tileset(ts, order=2)
        g.set_host_layout(layout)
        perm = g.tile_order()
        assert sorted(perm.tolist()) == list(range(mp))
        outs = []
        for k in range(n):
            f = np.ascontiguousarray(F[k] if layout == 0 else F[k][:, perm])
            out = np.empty((8, mp), np.float32)
            g.step_host(k + 1, f, out, ts.dels)
            g.synchronize()
            outs.append(out if layout == 0 else out[:, np.argsort(perm)])   # back to caller order
        runs.append((outs, {k: g.get(k) for k in ("wb", "tgg", "snowd", "cansto", "out")}))
        g.close()
    (o0, s0), (o1, s1) = runs
    for k in range(n):
        np.testing.assert_array_equal(o1[k], o0[k], err_msg="step %d" % k)
    for k in s0:
        np.testing.assert_array_equal(s1[k], s0[k], err_msg=k)


def test_config2_full_size_against_fp64_oracle(runtime):
    """The gridded workload at its full size, 1,000,000 tiles x 48 steps, on
    the benchmarked kernels (diagnostics off), against the FP64 oracle on the
    GPU's own forcing: every output every step and the soil profiles at the
    end, each held to harness.noise_criterion against the reference's own
    REAL = FP32 / r_2 = FP64 build on the same inputs."""
    import parity_full as P
    rep = P.config2_report(mp=1_000_000, nsteps=48)
    bad = {}
    for k, r in rep["fields"].items():
        g, m = r["gpu"], r["precision_mix"]
        assert "nonfinite" not in g, (k, g)
        if r["tol"] is not None:
            bad[k] = H.noise_criterion(g, m)
    assert not any(bad.values()), {k: (v, rep["fields"][k]) for k, v in bad.items() if v}
