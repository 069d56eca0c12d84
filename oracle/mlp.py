"""CPU restatement of the learned parameter proposal's network (forward, backward, Adam).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA kernels in
sdpa-gmp_gb300/csrc/mlp.cu; never part of the product path.

The network has no counterpart in the reference solver (its lambdaStar and
betaStar/betaBar are constants of param.sdpa).  Layout, as in include/sdpg.h:
flat parameters W1[64][6] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[2][64] b4[2]
(row-major [out][in]); scaling x_mean[6] x_std[6] y_mean[2] y_std[2].  Hidden layers
use tanh; the output layer is linear.  The loss of a batch of B samples is
    sum_{i,o} mask[i,o] * (z[i,o] - (t[i,o] - y_mean[o]) / y_std[o])**2 / B
in standardised output units.  Everything here runs in float64, so the finite-
difference check of the analytic gradient is tight.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 6, 64, 2
SHAPES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
          ("W4", (OUT, H)), ("b4", (OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)
N_SCALE = 2 * IN + 2 * OUT


def unpack(w: np.ndarray) -> dict:
    w = np.asarray(w, dtype=np.float64)
    out, off = {}, 0
    for name, shape in SHAPES:
        k = int(np.prod(shape))
        out[name] = w[off:off + k].reshape(shape)
        off += k
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def _split_scale(sc: np.ndarray):
    sc = np.asarray(sc, dtype=np.float64)
    return sc[:IN], sc[IN:2 * IN], sc[2 * IN:2 * IN + OUT], sc[2 * IN + OUT:]


def forward(w: np.ndarray, sc: np.ndarray, x: np.ndarray, cache: bool = False):
    """De-standardised outputs y[B][2] (and the activations if cache)."""
    p = unpack(w)
    xm, xs, ym, ys = _split_scale(sc)
    a0 = (np.asarray(x, dtype=np.float64) - xm) / xs
    a1 = np.tanh(a0 @ p["W1"].T + p["b1"])
    a2 = np.tanh(a1 @ p["W2"].T + p["b2"])
    a3 = np.tanh(a2 @ p["W3"].T + p["b3"])
    z = a3 @ p["W4"].T + p["b4"]
    y = ym + ys * z
    if cache:
        return y, (a0, a1, a2, a3, z)
    return y


def loss_and_grad(w: np.ndarray, sc: np.ndarray, x: np.ndarray, t: np.ndarray, mask: np.ndarray):
    """The batch loss above and its gradient with respect to the flat parameters."""
    p = unpack(w)
    _, _, ym, ys = _split_scale(sc)
    _, (a0, a1, a2, a3, z) = forward(w, sc, x, cache=True)
    B = z.shape[0]
    e = z - (np.asarray(t, dtype=np.float64) - ym) / ys
    m = np.asarray(mask, dtype=np.float64)
    loss = float(np.sum(m * e * e) / B)
    d4 = 2.0 * m * e / B
    g = {"W4": d4.T @ a3, "b4": d4.sum(0)}
    d3 = (d4 @ p["W4"]) * (1.0 - a3 * a3)
    g["W3"], g["b3"] = d3.T @ a2, d3.sum(0)
    d2 = (d3 @ p["W3"]) * (1.0 - a2 * a2)
    g["W2"], g["b2"] = d2.T @ a1, d2.sum(0)
    d1 = (d2 @ p["W2"]) * (1.0 - a1 * a1)
    g["W1"], g["b1"] = d1.T @ a0, d1.sum(0)
    return loss, pack(g)


def finite_difference(w, sc, x, t, mask, index: np.ndarray, h: float = 1e-6) -> np.ndarray:
    """Central differences of the loss at the listed parameter indices."""
    w = np.asarray(w, dtype=np.float64)
    out = np.zeros(len(index))
    for k, i in enumerate(index):
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        out[k] = (loss_and_grad(wp, sc, x, t, mask)[0] - loss_and_grad(wm, sc, x, t, mask)[0]) / (2 * h)
    return out


def adam_step(w, g, m1, m2, step: int, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
    """One Adam update (Kingma & Ba 2015); returns (w, m1, m2)."""
    m1 = b1 * m1 + (1 - b1) * g
    m2 = b2 * m2 + (1 - b2) * g * g
    w = w - lr * (m1 / (1 - b1 ** step)) / (np.sqrt(m2 / (1 - b2 ** step)) + eps)
    return w, m1, m2


def glorot_params(seed: int) -> np.ndarray:
    """Random parameters for tests (Glorot-uniform weights, small random biases)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if len(shape) == 2:
            a = np.sqrt(6.0 / (shape[0] + shape[1]))
            d[name] = rng.uniform(-a, a, shape)
        else:
            d[name] = rng.uniform(-0.1, 0.1, shape)
    return pack(d)
