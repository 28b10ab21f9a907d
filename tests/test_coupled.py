"""The coupled (ACCESS) calls of the oracle, against the structure of
src/coupled/AM3/control/cable/CM3/cbl_cbm_mod.F90 and the implicit driver's
prognostic bank (cable_implicit_main.F90:190-213, cbl_prognostic_bank.F90):

- cbm_expl runs the same define_canopy as the offline cbm() and leaves the
  prognostic state as it was but for rtsoil, ga and the carried LAI;
- an implicit cycle that is not the last reinstates the banked fields
  exactly and leaves the balance totals alone;
- the last implicit cycle advances soil and snow exactly as the offline step
  does, and its radiative temperature carries the start-of-step surface
  temperature and (l_rev_corr) the same correction fns_cor that rnet gets."""
import numpy as np
import pytest

import oracle_lib as O
from cable_gb300 import workloads as W

LAKES = 16
BANKED = ["wb", "wbice", "tgg", "tggsn", "ssdn", "smass", "sdepth", "isflag", "snowd", "ssdnn", "snage", "pudsto",
          "rtsoil", "owetfac", "wb_lake", "tss", "cansto", "cplant", "csoil"]
SIGMA = 5.67e-8


@pytest.fixture(scope="module")
def spun_up():
    """A snow-covered grid after 12 offline steps, and the forcing of step 13."""
    ts = W.snow_grid(600, seed=31, nsteps=16)
    st = O.init_state(ts)
    O.run(ts, st, 12)
    return ts, st, O.forcing(ts, 12, 1)


def _split(st):
    return {k: np.array(v) for k, v in O.split_state(st).items()}


def test_explicit_call_leaves_state_and_matches_offline_canopy(spun_up):
    ts, st0, F = spun_up
    st = st0.copy()
    d = O.run_calls(ts, st, [(13, 1, 1, 1)], forcing=F)
    a, b = _split(st0), _split(st)
    for k in a:
        if k in ("rtsoil", "ga", "vlaiw"):
            continue
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    assert np.array_equal(b["vlaiw"][0], d["vlaiw"])       # lai_refresh stores the LAI it used
    # radiative temperature from the start-of-step surface temperature
    np.testing.assert_allclose(d["trad"] ** 4, (1 - d["transd"]) * d["tv"] ** 4 + d["transd"] * a["tss"][0] ** 4,
                               rtol=1e-12)
    # the same canopy as the offline step on non-lake tiles (the offline
    # driver's lakes fix changes the top-layer water before the canopy)
    st2 = st0.copy()
    d2 = O.run(ts, st2, 1, ktau0=13, forcing=F)
    m = np.asarray(ts.iveg) != LAKES
    for k in ("fe", "fh", "tv", "rnet", "ga", "fpn", "frday", "fgpp", "rtsoil"):
        x = d[k] if k != "rtsoil" else b["rtsoil"][0]
        y = d2[k] if k != "rtsoil" else _split(st2)["rtsoil"][0]
        np.testing.assert_array_equal(x[m], y[m], err_msg=k)
    # without lai_refresh the carried LAI is used as it is
    st3 = st.copy()
    carried = 0.5 * b["vlaiw"][0]
    O.split_state(st3)["vlaiw"][0] = carried   # a view into st3
    d3 = O.run_calls(ts, st3, [(13, 1, 1, 0)], forcing=F)
    np.testing.assert_array_equal(d3["vlaiw"], carried)


def test_nonfinal_implicit_cycle_reinstates_the_bank(spun_up):
    ts, st0, F = spun_up
    st = st0.copy()
    O.run_calls(ts, st, [(13, 1, 1, 1)], forcing=F)
    mid = _split(st)
    d = O.run_calls(ts, st, [(13, 2, 0, 0)], forcing=F)
    after = _split(st)
    for k in BANKED + ["owb", "ebal_tot", "wbal_tot", "vlaiw", "first_call"]:
        np.testing.assert_array_equal(after[k], mid[k], err_msg=k)
    # not in the bank: the layer heat capacities soil_snow recomputed
    assert not np.array_equal(after["gammzz"], mid["gammzz"])
    # the cycle still produced its fluxes; tss was reset, so trad carries
    # only the start-of-step temperature
    np.testing.assert_allclose(d["trad"] ** 4, (1 - d["transd"]) * d["tv"] ** 4 + d["transd"] * mid["tss"][0] ** 4,
                               rtol=1e-12)


@pytest.mark.parametrize("rev_corr", [False, True])
def test_final_implicit_call_advances_like_offline(spun_up, rev_corr):
    ts, st0, F = spun_up
    sw = {"l_rev_corr": rev_corr}
    st = st0.copy()
    O.run_calls(ts, st, [(13, 1, 1, 1)], forcing=F, **sw)
    pre = st.copy()
    d = O.run_calls(ts, st, [(13, 2, 1, 0)], forcing=F, **sw)
    st2 = pre.copy()
    d2 = O.run(ts, st2, 1, ktau0=13, forcing=F, **sw)
    a, b, p = _split(st), _split(st2), _split(pre)
    m = np.asarray(ts.iveg) != LAKES
    # soil, snow and carbon advance exactly as in the offline step
    for k in ("wb", "wbice", "tgg", "tggsn", "ssdn", "smass", "sdepth", "isflag", "snowd", "ssdnn", "snage",
              "pudsto", "tss", "cansto", "owetfac", "cplant", "csoil"):
        np.testing.assert_array_equal(a[k][:, m], b[k][:, m], err_msg=k)
    # no balance checks in the coupled calls
    for k in ("owb", "ebal_tot", "wbal_tot"):
        np.testing.assert_array_equal(a[k], p[k], err_msg=k)
    for k in ("tv", "fpn", "frday", "fgpp"):
        np.testing.assert_array_equal(d[k][m], d2[k][m], err_msg=k)
    # the corrections: fh moves with the surface temperature change and the
    # melt, fe likewise; rnet and ga only under l_rev_corr
    fns_cor = d["rnet"] - d2["rnet"]
    if not rev_corr:
        np.testing.assert_array_equal(d["rnet"][m], d2["rnet"][m])
        np.testing.assert_array_equal(d["ga"][m], d2["ga"][m])
    else:
        assert np.abs(fns_cor[m]).max() > 0.0
    dts = a["tss"][0] - p["tss"][0]
    moved = m & (np.abs(dts) > 1e-3)
    assert moved.sum() > 50
    assert np.abs(d["fh"] - d2["fh"])[moved].max() > 0.0
    # trad: start-of-step temperature plus fns_cor / sigma
    np.testing.assert_allclose(d["trad"][m] ** 4, ((1 - d["transd"]) * d["tv"] ** 4 + d["transd"] * p["tss"][0] ** 4
                                                    + fns_cor / SIGMA)[m], rtol=1e-9, atol=1e-3)
