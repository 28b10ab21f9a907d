"""CPU oracle self-tests: closed-form unit checks and physical invariants.

The reference ships no golden vectors for the cbm() path and its Fortran
cannot be compiled here, so the oracle is pinned by these invariants and by
its own committed fixtures (tests/golden)."""
import numpy as np
import pytest

from cable_gb300 import workloads as W


def test_stability_functions_vanish_at_neutral(oracle):
    L = oracle.lib()
    assert L.cbmref_psim(0.0) == pytest.approx(0.0, abs=1e-12)
    assert L.cbmref_psis(0.0) == pytest.approx(0.0, abs=1e-12)
    # continuity across zeta = 0 and the unstable closed forms
    assert abs(L.cbmref_psim(1e-6) - L.cbmref_psim(-1e-6)) < 1e-4
    x = (1 + 16 * 2.0) ** 0.25
    ref = np.log((1 + x * x) * (1 + x) ** 2 / 8) - 2 * np.arctan(x) + 3.1415927 / 2
    assert L.cbmref_psim(-2.0) == pytest.approx(ref, rel=1e-12)
    y = (1 + 16 * 2.0) ** 0.5
    assert L.cbmref_psis(-2.0) == pytest.approx(2 * np.log((1 + y) / 2), rel=1e-12)


def test_qsat_matches_magnus(oracle):
    L = oracle.lib()
    for tc in (-20.0, 0.0, 15.0, 35.0):
        es = 6.106 * np.exp(17.27 * tc / (237.3 + tc))
        assert L.cbmref_qsat(tc, 1000.0) == pytest.approx(0.018016 / 0.02897 * es / 1000.0, rel=1e-12)


def test_spitter_pieces(oracle):
    L = oracle.lib()
    assert L.cbmref_spitter(100, 0.5, 5.0) == 0.0          # fsd below 10 W/m2
    assert L.cbmref_spitter(100, 1e-12, 500.0) == 0.0      # sun below horizon
    f = [L.cbmref_spitter(180, cz, 900.0 * cz) for cz in (0.2, 0.5, 0.9)]
    assert all(0.0 <= v <= 1.0 for v in f)


def test_trimb_matches_dense_solve(oracle):
    import ctypes as C
    L = oracle.lib()
    rng = np.random.default_rng(0)
    for n in (6, 9):
        a = -rng.uniform(0, 2, n); c = -rng.uniform(0, 2, n)
        a[0] = 0.0; c[-1] = 0.0
        b = 1.0 - a - c + rng.uniform(0, 1, n)
        r = rng.normal(size=n)
        M = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
        x = np.linalg.solve(M, r)
        rr = r.copy()
        dp = lambda v: v.ctypes.data_as(C.POINTER(C.c_double))
        L.cbmref_trimb(dp(a), dp(b), dp(c), dp(rr), n)
        np.testing.assert_allclose(rr, x, rtol=1e-12, atol=1e-12)


def test_photosynthesis_is_limited_by_its_rubisco_root(oracle):
    """The returned assimilation is the minimum of three limits; check it
    never exceeds the Rubisco-limited rate computed from the quadratic."""
    L = oracle.lib()
    rng = np.random.default_rng(1)
    for _ in range(200):
        csx = rng.uniform(2e-4, 5e-4); cx1 = rng.uniform(3e-4, 8e-4); cx2 = rng.uniform(5e-5, 1e-4)
        gswmin = 0.01; rdx = rng.uniform(0, 1e-6); v3 = rng.uniform(1e-6, 6e-5); v4 = 0.0
        vx3 = rng.uniform(1e-6, 6e-5); vx4 = 0.0; gs = rng.uniform(1e3, 3e4); fw = rng.uniform(0.2, 1)
        an = L.cbmref_photosynthesis(csx, cx1, cx2, gswmin, rdx, v3, v4, vx3, vx4, gs, fw)
        g = gswmin * fw / 1.57
        c2 = g + gs * (v3 - (rdx - v4))
        c1 = (1 - csx * gs) * (v3 + v4 - rdx) + g * (cx1 - csx) - gs * (v3 * cx2 / 2 + cx1 * (rdx - v4))
        c0 = -(1 - csx * gs) * (v3 * cx2 / 2 + cx1 * (rdx - v4)) - g * cx1 * csx
        ci = max(0.0, (-c1 + np.sqrt(max(0.0, c1 * c1 - 4 * c0 * c2))) / (2 * c2))
        assert c2 * ci * ci + c1 * ci + c0 == pytest.approx(0.0, abs=1e-9 * max(1.0, abs(c1)) + 1e-14)
        arub = v3 * (ci - cx2 / 2) / (ci + cx1) + v4 - rdx
        assert an <= arub + 1e-15


def _run(oracle, ts, steps, precision=0):
    st = oracle.init_state(ts, precision)
    d = oracle.run(ts, st, steps, precision=precision)
    return oracle.split_state(st), d


def test_site_energy_and_leaf_balance_close(oracle):
    ts = W.site5(nsteps=96)
    S, d = _run(oracle, ts, 96)
    assert np.all(np.abs(d["ebal"]) < 1e-9)      # cable_checks.F90 energy_balance
    assert np.all(np.abs(d["drybal"]) < 1e-8)    # leaf energy balance at convergence
    assert np.all(np.abs(d["wbal"]) < 1e-8)      # mass_balance (no puddles / lakes here)
    assert np.all(np.abs(S["ebal_tot"]) < 1e-7)


def test_grid_energy_closure_and_ranges(oracle):
    ts = W.snow_grid(3000, nsteps=24)
    S, d = _run(oracle, ts, 24)
    for k, v in d.items():
        assert np.all(np.isfinite(v)), k
    assert np.abs(d["ebal"]).max() < 1e-8
    # cable_checks.F90 range checks
    assert d["tv"].min() > 213 and d["tv"].max() < 333
    assert S["tgg"].min() > 200 and S["tgg"].max() < 350
    assert np.all(S["wb"] >= 0) and np.all(S["wb"] <= 0.5)
    assert np.all(d["fwsoil"] >= 0) and np.all(d["fwsoil"] <= 1)
    assert d["dryleaf_passes"].max() <= 4 * 20
    assert set(np.unique(S["isflag"])) <= {0.0, 1.0}


def test_water_balance_closes_where_the_reference_conserves(oracle):
    """mass_balance (cable_checks.F90:472-551) omits puddle storage; with that
    added the budget closes to round-off except where the reference itself
    leaks: the frozen-soil ice cap in soilfreeze (cbl_soilfreeze.F90:36-39
    caps wbice but not wb) and a stale evapfbl when dryLeaf's best iterate
    condenses (cbl_dryLeaf.F90:613-657 restores it only for ecy > 0)."""
    ts = W.grid(4000, nsteps=36)
    st = oracle.init_state(ts)
    oracle.run(ts, st, 35)
    p0 = oracle.split_state(st)["pudsto"][0].copy()
    d = oracle.run(ts, st, 1, ktau0=36)
    S = oracle.split_state(st)
    r = np.abs(d["wbal"] - (S["pudsto"][0] - p0))
    unfrozen = ~(S["wbice"] > 0).any(0)
    nl = (ts.iveg != 16) & unfrozen
    assert (r[nl] < 1e-9).mean() > 0.98
    assert r[nl].max() < 1e-3


def test_reference_precision_mix_tracks_fp64(oracle):
    """<float,double> (the reference's own REAL/r_2 mix) against the FP64
    oracle: the reference's precision noise floor."""
    ts = W.grid(2000, nsteps=24)
    S64, d64 = _run(oracle, ts, 24, 0)
    S32, d32 = _run(oracle, ts, 24, 1)
    for k, tol in (("fe", 1.0), ("fh", 1.0), ("tv", 0.01)):
        e = d32[k] - d64[k]
        assert np.sqrt(np.mean(e * e)) < tol, k
    e = S32["tgg"] - S64["tgg"]
    assert np.sqrt(np.mean(e * e)) < 0.01


def test_oracle_is_deterministic_and_thread_count_independent(oracle):
    ts = W.grid(500, nsteps=6)
    a = oracle.init_state(ts); b = oracle.init_state(ts)
    oracle.run(ts, a, 6, nthreads=1)
    oracle.run(ts, b, 6, nthreads=4)
    assert np.array_equal(a, b)


def test_restart_continuation_is_bitwise(oracle):
    """Advancing 12 steps equals 6 + 6 steps from the saved state."""
    ts = W.snow_grid(400, nsteps=12)
    a = oracle.init_state(ts)
    oracle.run(ts, a, 12)
    b = oracle.init_state(ts)
    oracle.run(ts, b, 6)
    saved = b.copy()
    oracle.run(ts, saved, 6, ktau0=7)
    assert np.array_equal(a, saved)


def test_forcing_generator_statistics(oracle):
    ts = W.grid(4000, nsteps=48)
    F = oracle.forcing(ts, 0, 48)
    names = oracle.FORCING_FIELDS
    f = dict(zip(names, np.moveaxis(F, 1, 0)))
    assert np.all(f["fsd1"] >= 0) and np.array_equal(f["fsd1"], f["fsd2"])
    wet = f["precip"] > 0
    assert 0.04 < wet.mean() < 0.06
    assert f["precip"][wet].mean() == pytest.approx(2.0, rel=0.1)
    assert np.all(f["precip_sn"][f["tk"] > 273.16] == 0)
    assert f["fld"].mean() == pytest.approx(300.0, abs=2.0)
    assert f["ua"].mean() == pytest.approx(3.0, rel=0.05)
    assert np.all((f["qv"] > 0) & (f["qv"] < 0.2))
    assert np.all((f["hod"] >= 0) & (f["hod"] < 24))
    # same seed -> same forcing
    assert np.array_equal(F, oracle.forcing(ts, 0, 48))


def test_soil_thermal_fix_switch_is_live_and_conserves(oracle):
    """With soil_thermal_fix the soil temperatures follow the new
    conductivity and heat-capacity parameters (the switch changes them), and
    the energy and leaf balances still close every step."""
    ts = W.snow_grid(mp=400, nsteps=48)
    res = {}
    for fix in (False, True):
        st = oracle.init_state(ts, 0)
        d = oracle.run(ts, st, 48, soil_thermal_fix=fix)
        res[fix] = (oracle.split_state(st), d)
    (s0, d0), (s1, d1) = res[False], res[True]
    assert np.abs(d1["ebal"]).max() < 1e-8
    assert np.abs(d1["drybal"]).max() < 1e-6
    dt = np.abs(np.asarray(s1["tgg"]) - np.asarray(s0["tgg"]))
    assert dt.max() > 0.05                       # the switch changes soil temperatures
    assert np.isfinite(np.asarray(s1["tgg"])).all()
    assert 200.0 < np.asarray(s1["tgg"]).min() and np.asarray(s1["tgg"]).max() < 340.0


SWITCH_CASES = {
    # switch set, diagnostic or state field the switch must move, threshold
    "litter": (dict(litter=True), "fhs", 1.0),
    "l_rev_corr": (dict(l_rev_corr=True), "tgg", 0.01),
    "fwsoil_nonlinear": (dict(fwsoil_switch="non-linear extrapolation"), "fevc", 1.0),
    "fwsoil_lai_ktaul": (dict(fwsoil_switch="Lai and Ktaul 2000"), "fevc", 1.0),
    "potev_pm": (dict(ssnow_potev="P-M"), "fes", 1.0),
    "reduce_soilevp": (dict(l_new_reduce_soilevp=True), "fes", 1.0),
    "runoff_speed": (dict(l_new_runoff_speed=True), "wb", 1e-4),
    "soil_resp_off": (dict(diag_soil_resp="OFF"), "frs", 1e-8),
}


@pytest.mark.parametrize("case", list(SWITCH_CASES))
def test_canopy_and_soil_switches_are_live_and_conserve(oracle, case):
    """Each alternative science switch changes what it should (the named
    field moves by more than the threshold over 48 steps of snowy gridded
    tiles) and the energy and leaf balances still close every step."""
    sw, field, thr = SWITCH_CASES[case]
    ts = W.snow_grid(mp=400, nsteps=48)
    res = {}
    for on in (False, True):
        st = oracle.init_state(ts, 0)
        d = oracle.run(ts, st, 48, **(sw if on else {}))
        res[on] = (oracle.split_state(st), d)
    (s0, d0), (s1, d1) = res[False], res[True]
    assert np.abs(d1["ebal"]).max() < 1e-8
    assert np.abs(d1["drybal"]).max() < 1e-6
    a0 = np.asarray(s0[field] if field in s0 else d0[field], np.float64)
    a1 = np.asarray(s1[field] if field in s1 else d1[field], np.float64)
    assert np.all(np.isfinite(a1))
    assert np.abs(a1 - a0).max() > thr, (case, np.abs(a1 - a0).max())


def test_switch_mask_rejects_unknown_values():
    from cable_gb300 import runtime as R
    assert R.switch_mask() == 0
    assert R.switch_mask(fwsoil_switch="Lai and Ktaul 2000", ssnow_potev="P-M", diag_soil_resp="OFF ") == 32 | 64 | 512
    for bad in (dict(fwsoil_switch="Haverd2013"), dict(ssnow_potev="PM"), dict(diag_soil_resp="maybe")):
        with pytest.raises(ValueError):
            R.switch_mask(**bad)
