"""FP64 numpy restatement of the dryLeaf surrogate network, the CPU
reference its GPU training and inference kernels are checked against.

Network: 12 normalised inputs -> 64 (SiLU) -> 64 (SiLU) -> 3 normalised
outputs.  Weights follow the GPU layout: W1 [64][12], W2 [64][64], W3
[3][64], biases b1 [64], b2 [64], b3 [3].  Loss: mean squared error over
the batch and the 3 outputs.  The GPU rounds inputs, weights and hidden
activations to BF16 and accumulates in FP32; ``quantise=True`` applies the
same BF16 rounding here so forward values can be compared tightly."""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 12, 64, 3


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init(seed=0):
    """He-style initial weights (the GPU trainer's initialisation is
    seeded separately; tests pass weights explicitly)."""
    rng = np.random.default_rng(seed)
    return {
        "W1": rng.standard_normal((NH, NIN)) * np.sqrt(2.0 / NIN), "b1": np.zeros(NH),
        "W2": rng.standard_normal((NH, NH)) * np.sqrt(2.0 / NH), "b2": np.zeros(NH),
        "W3": rng.standard_normal((NOUT, NH)) * np.sqrt(1.0 / NH), "b3": np.zeros(NOUT),
    }


def forward(p, x, quantise=False):
    q = bf16 if quantise else (lambda a: np.asarray(a, np.float64))
    W1, W2, W3 = q(p["W1"]), q(p["W2"]), q(p["W3"])
    a0 = q(x)
    z1 = a0 @ W1.T + p["b1"]
    a1 = q(silu(z1))
    z2 = a1 @ W2.T + p["b2"]
    a2 = q(silu(z2))
    y = a2 @ W3.T + p["b3"]
    return y, {"a0": a0, "z1": z1, "a1": a1, "z2": z2, "a2": a2, "W1": W1, "W2": W2, "W3": W3}


def loss_and_grads(p, x, t, quantise=False):
    y, c = forward(p, x, quantise)
    n = x.shape[0]
    d = y - t
    loss = float(np.mean(d * d))
    dy = 2.0 * d / (n * NOUT)
    g = {"W3": dy.T @ c["a2"], "b3": dy.sum(0)}
    dz2 = (dy @ c["W3"]) * dsilu(c["z2"])
    g["W2"] = dz2.T @ c["a1"]
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ c["W2"]) * dsilu(c["z1"])
    g["W1"] = dz1.T @ c["a0"]
    g["b1"] = dz1.sum(0)
    return loss, g


def adam_step(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015, bias-corrected), in place."""
    for k in p:
        m[k] = b1 * m[k] + (1 - b1) * g[k]
        v[k] = b2 * v[k] + (1 - b2) * g[k] * g[k]
        mh = m[k] / (1 - b1 ** step)
        vh = v[k] / (1 - b2 ** step)
        p[k] = p[k] - lr * mh / (np.sqrt(vh) + eps)
