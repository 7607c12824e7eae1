"""CPU oracle of the learned (a, b) proposal -- TEST INFRASTRUCTURE ONLY.

FP64 NumPy restatement of what the CUDA kernels in
fastfuncstuff_gb300/csrc/learned.cu compute, used by the tests to check them:

* features: the OLS residual's autocorrelations at lags 1-8, each the sum of
  lag-k products inside runs over the residual's sum of squares, plus T/1000;
* the MLP 9 -> 64 -> 64 -> 2 with exact (erf) GELU, its mean-squared-error loss
  L = sum (out - y)^2 / (2 B) and the gradients of L;
* one Adam step.

The proposal has no counterpart in the reference (it is this build's learned
seed for the grid search); the oracle is the mathematics written out, nothing
more.
"""

from __future__ import annotations

import math

import numpy as np

N_IN, N_H, N_OUT = 9, 64, 2
SHAPES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)),
          ("W3", (N_OUT, N_H)), ("b3", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[o : o + n], np.float64).reshape(shape)
        o += n
    return out


def init(seed: int = 0) -> np.ndarray:
    """He-style initial weights, zero biases (float32 flat vector)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SHAPES:
        if name.startswith("W"):
            parts.append(rng.standard_normal(shape).ravel() * math.sqrt(2.0 / shape[1]))
        else:
            parts.append(np.zeros(shape).ravel())
    return np.concatenate(parts).astype(np.float32)


def features(yr: np.ndarray, run_start, n_lags: int = 8) -> np.ndarray:
    """(V, 9) lag-1..8 autocorrelations of each row (within runs) and T/1000."""
    yr = np.asarray(yr, np.float64)
    V, T = yr.shape
    rs = list(np.asarray(run_start).reshape(-1))
    if rs[-1] != T:
        rs = rs + [T]
    s0 = (yr * yr).sum(1)
    out = np.zeros((V, n_lags + 1))
    for k in range(1, n_lags + 1):
        acc = np.zeros(V)
        for r in range(len(rs) - 1):
            a, b = rs[r], rs[r + 1]
            if b - a > k:
                acc += (yr[:, a : b - k] * yr[:, a + k : b]).sum(1)
        out[:, k - 1] = np.where(s0 > 0, acc / np.where(s0 > 0, s0, 1.0), 0.0)
    out[:, n_lags] = T / 1000.0
    return out


def _gelu(z):
    from scipy.special import erf

    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def _gelu_grad(z):
    from scipy.special import erf

    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(flat: np.ndarray, x: np.ndarray) -> np.ndarray:
    p = unpack(flat)
    h1 = _gelu(np.asarray(x, np.float64) @ p["W1"].T + p["b1"])
    h2 = _gelu(h1 @ p["W2"].T + p["b2"])
    return h2 @ p["W3"].T + p["b3"]


def loss_and_grad(flat: np.ndarray, x: np.ndarray, y: np.ndarray, n_total: int | None = None):
    """L = sum (out - y)^2 / (2 n_total) and dL/dparams (flat, float64)."""
    p = unpack(flat)
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = n_total or x.shape[0]
    z1 = x @ p["W1"].T + p["b1"]
    h1 = _gelu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = _gelu(z2)
    out = h2 @ p["W3"].T + p["b3"]
    e = out - y
    loss = (e * e).sum() / (2.0 * n)
    d_out = e / n
    g = {"W3": d_out.T @ h2, "b3": d_out.sum(0)}
    dz2 = (d_out @ p["W3"]) * _gelu_grad(z2)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * _gelu_grad(z1)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SHAPES])


def adam(flat, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected); returns new (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1**step)
    vh = v / (1 - b2**step)
    return flat - lr * mh / (np.sqrt(vh) + eps), m, v
