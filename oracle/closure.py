"""TEST INFRASTRUCTURE — float64 numpy restatement of the learned closure's network, the oracle
of the CUDA training kernels (lbm_mlp_forward / lbm_mlp_backward / lbm_mlp_adam).

Only tests/ import this module.  The network is 8 -> 32 -> 32 -> 1 with ReLU hidden layers and
a softplus output scaled by nu_scale; theta packs w1 (8x32, input-major), b1, w2 (32x32), b2,
w3 (32), b3 — 1377 parameters.  No counterpart in the reference (its LES is Smagorinsky only).
"""
from __future__ import annotations

import numpy as np

SIZES = (("w1", (8, 32)), ("b1", (32,)), ("w2", (32, 32)), ("b2", (32,)), ("w3", (32,)), ("b3", ()))
N_PARAMS = 1377


def unpack(theta):
    t = np.asarray(theta, dtype=np.float64).ravel()
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape)) if shape else 1
        out[name] = t[o:o + n].reshape(shape) if shape else t[o]
        o += n
    return out


def pack(p) -> np.ndarray:
    return np.concatenate([np.ravel(np.asarray(p[name], dtype=np.float64)) for name, _ in SIZES])


def softplus(y):
    return np.where(y > 20, y, np.log1p(np.exp(np.minimum(y, 20))))


def forward(theta, x, nu_scale: float):
    """nu (n,) and the activations the backward pass needs."""
    p = unpack(theta)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ p["w1"] + p["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ p["w2"] + p["b2"]
    h2 = np.maximum(a2, 0)
    y = h2 @ p["w3"] + p["b3"]
    return softplus(y) * nu_scale, (x, h1, h2, y)


def backward(theta, x, g, nu_scale: float) -> np.ndarray:
    """d(sum_i g_i nu_i) / d theta, packed like theta."""
    p = unpack(theta)
    _, (x, h1, h2, y) = forward(theta, x, nu_scale)
    gy = np.asarray(g, dtype=np.float64) * nu_scale / (1 + np.exp(-y))
    dh2 = np.outer(gy, p["w3"]) * (h2 > 0)
    dh1 = (dh2 @ p["w2"].T) * (h1 > 0)
    return pack({"w1": x.T @ dh1, "b1": dh1.sum(0), "w2": h1.T @ dh2, "b2": dh2.sum(0), "w3": h2.T @ gy,
                 "b3": gy.sum()})


def adam(theta, grad, m, v, lr, beta1, beta2, eps, t):
    """One Adam step (Kingma & Ba, ICLR 2015, Algorithm 1); returns new theta, m, v."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
