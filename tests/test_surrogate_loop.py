"""The dryLeaf surrogate end to end on the GPU: harvest training rows from
the plain kernel, train the network with the library's own tensor-core
kernels, run the timestep with the network in the loop, and compare with
the method without it (the plain iteration's usual start, which a network
predicting no change reproduces) and with the FP64 oracle (latent heat RMSE
at most 2 W/m2, canopy temperature RMSE at most 0.05 K)."""
import numpy as np
import pytest

import harness as H
from cable_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    from cable_gb300 import runtime as R
    ts = W.snow_grid(20000, seed=31, nsteps=96)
    g = R.from_tileset(ts)
    n = g.harvest(1, 96, prob=0.2, seed=5)
    rows = g.harvest_rows(n)
    losses = g.surrogate_train(epochs=12, batch=8192, lr=2e-3, val_frac=0.1, seed=2)
    params, norm = g.surrogate_weights()
    g.close()
    return rows, losses, params, norm


def test_harvest_rows_are_physical(trained):
    rows, _, _, _ = trained
    assert rows.shape[0] > 150_000
    assert np.all(np.isfinite(rows[:, :15]))
    assert rows[:, 0].min() > -10 and rows[:, 1].min() > -10               # absorbed PAR (W/m2; the
    # reference's shaded-leaf PAR can come out slightly negative at low sun)
    assert np.all((rows[:, 2] > 200) & (rows[:, 2] < 350))                 # leaf temperature at entry
    assert np.all(rows[:, 8] > 0) and np.all(rows[:, 8] <= 1)              # soil moisture stress
    assert np.all(rows[:, 12] >= 1e-3 - 1e-6)                              # gs floor of dryLeaf
    assert np.abs(rows[:, 14]).max() < 30                                  # leaf temperature change


def test_training_reduces_validation_error(trained):
    _, losses, _, _ = trained
    assert np.all(np.isfinite(losses))
    assert losses[-1, 1] < 0.5 * losses[0, 1] or losses[-1, 1] < 0.1, losses
    assert losses[-1, 1] < 0.5, losses


def _run(ts, params, norm, mode, nsteps):
    from cable_gb300 import runtime as R
    g = R.from_tileset(ts)
    g.set_options(diag=True, capture_forcing=True)
    if mode:
        g.surrogate_weights(params, norm)
        g.set_surrogate(mode, 0.1)
        g.surrogate_stats(reset=True)
    F, passes = [], 0.0
    for k in range(nsteps):
        g.step(1 + k)
        F.append(g.get("forcing"))
        passes += float(g.get("dryleaf_passes")[0].sum())
    g.synchronize()
    state = {k: g.get(k) for k in H.STATE_FIELDS}
    diag = {k: g.get(k)[0] for k in H.DIAG_MAP}
    stats = g.surrogate_stats() if mode else (0, 0)
    g.close()
    return state, diag, np.stack(F), passes, stats


def _zero_net(norm):
    """A network that predicts no leaf-temperature change: the iteration
    then starts where it starts without the surrogate."""
    from cable_gb300 import runtime as R
    z = np.zeros(R.MLP_NPARAM, np.float32)
    n = norm.copy()
    n[24:27] = 0.0
    return z, n


def test_network_gains_over_the_plain_start(trained):
    _, _, params, norm = trained
    ts = W.snow_grid(8000, seed=77, nsteps=24)          # other tiles and forcing than the training run
    _, _, _, p_net, (tried, acc) = _run(ts, params, norm, 1, 24)
    zp, zn = _zero_net(norm)
    _, _, _, p_zero, (tried0, acc0) = _run(ts, zp, zn, 1, 24)
    _, _, _, p_warm, _ = _run(ts, params, norm, 2, 24)
    _, _, _, p_plain, _ = _run(ts, params, norm, 0, 24)
    assert tried == tried0 > 0
    # one-pass closures of the first Monin-Obukhov iteration's dryLeaf
    assert acc > 2 * acc0, (acc, acc0, tried)
    # warm start: fewer dryLeaf passes than the plain iteration
    assert p_warm < p_plain, (p_warm, p_plain)
    # strict mode costs at most one extra pass per rejected prediction
    assert p_net <= p_plain + (tried - acc) + 1e-6


def test_strict_surrogate_error_against_fp64(oracle, trained):
    _, _, params, norm = trained
    ts = W.snow_grid(8000, seed=78, nsteps=48)
    s_sur, d_sur, F, _, (tried, acc) = _run(ts, params, norm, 1, 48)
    st = oracle.init_state(ts, 0)
    od = oracle.run(ts, st, 48, forcing=F, precision=0)
    e_le = np.sqrt(np.mean((d_sur["fe_d"] - od["fe"]) ** 2))
    e_tv = np.sqrt(np.mean((d_sur["tv_d"] - od["tv"]) ** 2))
    assert e_le <= 2.0, e_le
    assert e_tv <= 0.05, e_tv


def test_tensor_core_give_up_falls_back_and_is_reported(trained, monkeypatch):
    """The network kernels' bounded tensor-core waits.  With the debug wait
    limit CABLEGPU_DEBUG_TC_WAIT_NS=0 every first wait gives up at once: the
    inference kernel then waits, with its full limit, for the pass it issued,
    frees its tensor memory, marks every tile "no prediction" and flags the
    failure.  The canopy kernel runs the plain iteration (the step is bitwise
    the plain kernel's), cablegpu_synchronize reports the failure, and the
    context-free forward pass returns an error.  With the limit restored the
    next step uses the network again, so the tensor memory was freed."""
    from cable_gb300 import runtime as R
    rows, _, params, norm = trained
    ts = W.snow_grid(8000, seed=81, nsteps=2)
    plain = R.from_tileset(ts)
    plain.step(1)
    plain.synchronize()
    ref = {k: plain.get(k) for k in ("out", "wb", "tgg", "tggsn", "snowd", "cansto", "rtsoil")}
    plain.close()
    g = R.from_tileset(ts)
    g.surrogate_weights(params, norm)
    g.set_surrogate(1, 0.1)
    g.surrogate_stats(reset=True)
    monkeypatch.setenv("CABLEGPU_DEBUG_TC_WAIT_NS", "0")
    g.step(1)
    with pytest.raises(R.CableGPUError) as e:
        g.synchronize()
    assert e.value.code == -2 and "surrogate" in str(e.value), e.value
    assert g.surrogate_stats(reset=True)[0] == 0          # no tile started from a prediction
    for k, v in ref.items():
        np.testing.assert_array_equal(g.get(k), v, err_msg=k)
    with pytest.raises(R.CableGPUError):
        R.mlp_forward(params, norm, rows[:4096])
    monkeypatch.delenv("CABLEGPU_DEBUG_TC_WAIT_NS")
    g.step(2)
    g.synchronize()
    tried, _ = g.surrogate_stats(reset=True)
    assert tried > 0
    y = R.mlp_forward(params, norm, rows[:4096])
    assert np.all(np.isfinite(y))
    g.close()


def test_surrogate_error_against_fp64_every_step(oracle, trained):
    """The benchmark's error statement over a run rather than at its end:
    latent heat and canopy temperature of every tile-step of 96 half-hour
    steps on 8,000 snow tiles, strict surrogate against the FP64 oracle on
    the same forcing (RMSE at most 2 W/m2 and 0.05 K), beside the
    reference's own FP32 build against the same oracle."""
    from cable_gb300 import runtime as R
    _, _, params, norm = trained
    ts = W.snow_grid(8000, seed=79, nsteps=96)
    g = R.from_tileset(ts)
    g.set_options(diag=True, capture_forcing=True)
    g.surrogate_weights(params, norm)
    g.set_surrogate(1, 0.1)
    st64, st32 = oracle.init_state(ts, 0), oracle.init_state(ts, 1)
    se = {"sur_fe": 0.0, "sur_tv": 0.0, "mix_fe": 0.0, "mix_tv": 0.0}
    n = 0
    for k in range(96):
        g.step(1 + k)
        F = g.get("forcing")[None]
        fe, tv = g.get("fe_d")[0], g.get("tv_d")[0]
        d64 = oracle.run(ts, st64, 1, ktau0=1 + k, forcing=F, precision=0)
        d32 = oracle.run(ts, st32, 1, ktau0=1 + k, forcing=F, precision=1)
        se["sur_fe"] += float(np.sum((fe - d64["fe"]) ** 2))
        se["sur_tv"] += float(np.sum((tv - d64["tv"]) ** 2))
        se["mix_fe"] += float(np.sum((d32["fe"] - d64["fe"]) ** 2))
        se["mix_tv"] += float(np.sum((d32["tv"] - d64["tv"]) ** 2))
        n += fe.size
    g.synchronize()
    g.close()
    rmse = {k: np.sqrt(v / n) for k, v in se.items()}
    print("surrogate over 96 steps x 8000 tiles:", {k: round(v, 4) for k, v in rmse.items()})
    assert rmse["sur_fe"] <= 2.0, rmse
    assert rmse["sur_tv"] <= 0.05, rmse
