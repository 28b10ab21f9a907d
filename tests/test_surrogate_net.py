"""The surrogate network's tensor-core kernels against the FP64 numpy
restatement in tests/mlp_ref.py: forward values, loss gradients (the
gradient check of the training kernels) and a training run that must learn
a smooth function."""
import numpy as np
import pytest

import mlp_ref as M


def _rows(x, t):
    r = np.zeros((x.shape[0], 16), np.float32)
    r[:, :12] = x
    r[:, 12:15] = t
    return r


def _norm(x, t):
    sd_x = x.std(0)
    sd_t = t.std(0)
    return np.concatenate([x.mean(0), 1.0 / sd_x, t.mean(0), sd_t]).astype(np.float32)


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 12)) * rng.uniform(0.5, 3.0, 12) + rng.uniform(-2, 2, 12)
    xn = (x - x.mean(0)) / x.std(0)
    t = np.stack([np.sin(xn[:, 0]) + 0.5 * xn[:, 1] * xn[:, 2], np.tanh(xn[:, 3] - xn[:, 4]),
                  0.3 * xn[:, 5] ** 2 - xn[:, 6] + 0.1 * xn[:, 7]], 1)
    return x.astype(np.float32), (t * [2.0, 0.5, 3.0] + [1.0, -2.0, 0.0]).astype(np.float32)


def _normalised(nrm, x, t):
    xn = (x - nrm[:12]) * nrm[12:24]
    tn = (t - nrm[24:27]) / nrm[27:30]
    return xn.astype(np.float64), tn.astype(np.float64)


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = M.init(5)
    for k in p:
        p[k] = p[k] + 0.1 * rng.standard_normal(p[k].shape)
    x = rng.standard_normal((40, 12))
    t = rng.standard_normal((40, 3))
    _, g = M.loss_and_grads(p, x, t)
    for k in ("W1", "b2", "W3"):
        idx = tuple(rng.integers(0, s) for s in p[k].shape)
        q = {kk: vv.copy() for kk, vv in p.items()}
        h = 1e-6
        q[k][idx] += h
        lp, _ = M.loss_and_grads(q, x, t)
        q[k][idx] -= 2 * h
        lm, _ = M.loss_and_grads(q, x, t)
        assert abs((lp - lm) / (2 * h) - g[k][idx]) < 1e-6 * max(1.0, abs(g[k][idx]))


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0], np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12


@pytest.mark.gpu
def test_forward_matches_reference():
    from cable_gb300 import runtime as R
    x, t = _data(1000, 1)              # 1000 rows: the last 128-row tile is ragged
    nrm = _norm(x, t)
    p = M.init(7)
    for k in ("b1", "b2", "b3"):
        p[k] = 0.1 * np.random.default_rng(2).standard_normal(p[k].shape)
    y = R.mlp_forward(R.mlp_pack(p), nrm, _rows(x, t))
    xn, _ = _normalised(nrm, x, t)
    yn_ref, _ = M.forward(p, xn, quantise=True)
    yn = (y - nrm[24:27]) / nrm[27:30]
    err = np.abs(yn - yn_ref)
    assert err.max() < 0.02 * max(1.0, np.abs(yn_ref).max()), err.max()
    assert np.sqrt(np.mean(err ** 2)) < 3e-3


@pytest.mark.gpu
def test_gradient_matches_reference():
    from cable_gb300 import runtime as R
    x, t = _data(2000, 4)
    nrm = _norm(x, t)
    p = M.init(11)
    loss, g = R.mlp_grad(R.mlp_pack(p), nrm, _rows(x, t))
    xn, tn = _normalised(nrm, x, t)
    loss_ref, g_ref = M.loss_and_grads(p, xn, tn, quantise=True)
    assert abs(loss - loss_ref) < 1e-2 * loss_ref
    G = R.mlp_unpack(g)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        a, b = np.ravel(G[k]).astype(np.float64), np.ravel(g_ref[k])
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        assert rel < 0.03 and cos > 0.999, (k, rel, cos)


@pytest.mark.gpu
def test_training_learns_a_smooth_function():
    from cable_gb300 import runtime as R
    x, t = _data(120_000, 9)
    rows = _rows(x, t)
    p, nrm, losses = R.mlp_fit(rows, nval=20_000, epochs=8, batch=4096, lr=2e-3, seed=3)
    assert np.all(np.isfinite(losses))
    assert losses[-1, 1] < 0.05, losses            # normalised MSE; 1.0 = predicting the mean
    assert losses[-1, 0] < 0.5 * losses[0, 0]
    # the trained network's forward pass agrees with the reference on held-out rows
    xv, tv = x[-2000:], t[-2000:]
    y = R.mlp_forward(p, nrm, _rows(xv, tv))
    xn, _ = _normalised(nrm, xv, tv)
    yn_ref, _ = M.forward(R.mlp_unpack(p), xn, quantise=True)
    yn = (y - nrm[24:27]) / nrm[27:30]
    assert np.abs(yn - yn_ref).max() < 0.05
