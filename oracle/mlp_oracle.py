"""CPU oracle of the boundary network (test infrastructure only: used by tests to check the GPU
kernels, never by the product path).

Restates the network of the learned boundary -- 81 inputs, two hidden layers of 64 with the
tanh-form GELU, one output -- and its mean-squared-error gradient, with the same roundings as the GPU
kernels: inputs, W1, W2 and the first hidden activations rounded to BF16 (round to nearest
even), everything else in float64 here (FP32 on the GPU).  The BF16 rounding is passed through
as the identity in the backward pass, as the GPU does.  `fd_check` validates the backward
formulas against central differences with the rounding switched off.

Parameter layout: W1[64][81], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
from __future__ import annotations

import math

import numpy as np

N_IN, H = 81, 64
SHAPES = [("W1", (H, N_IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("w3", (H,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in SHAPES])


def bf16(a):
    """Round float32 values to BF16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_GC = math.sqrt(2.0 / math.pi)
_GA = 0.044715


def gelu(z):
    """GELU in the tanh form of Hendrycks & Gimpel (2016): z/2 (1 + tanh(sqrt(2/pi)(z + 0.044715 z^3)))."""
    return 0.5 * z * (1.0 + np.tanh(_GC * (z + _GA * z ** 3)))


def gelu_d(z):
    t = np.tanh(_GC * (z + _GA * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _GC * (1.0 + 3.0 * _GA * z * z)


def forward(p, x, rounding=True):
    d = unpack(p)
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    xb = r(x)
    W1, W2 = r(d["W1"]), r(d["W2"])
    z1 = xb @ W1.T + d["b1"]
    h1 = r(gelu(z1).astype(np.float32)) if rounding else gelu(z1)
    z2 = h1 @ W2.T + d["b2"]
    h2 = gelu(z2)
    y = h2 @ d["w3"] + d["b3"][0]
    return y, dict(xb=xb, W1=W1, W2=W2, z1=z1, h1=h1, z2=z2, h2=h2)


def loss_grad(p, x, t, rounding=True):
    """(mean squared error, gradient with respect to the parameters)."""
    y, c = forward(p, x, rounding)
    n = len(y)
    e = y - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    d = unpack(p)
    dy = 2.0 * e / n
    dz2 = dy[:, None] * d["w3"][None, :] * gelu_d(c["z2"])
    g = {"w3": c["h2"].T @ dy, "b3": np.array([dy.sum()]), "b2": dz2.sum(0), "W2": dz2.T @ c["h1"]}
    dh1 = dz2 @ c["W2"]
    dz1 = dh1 * gelu_d(c["z1"])
    g["b1"] = dz1.sum(0)
    g["W1"] = dz1.T @ c["xb"]
    return loss, pack(g)


def fd_check(seed=0, n=16, eps=1e-6, probes=24):
    """Largest relative error of the analytic gradient (no rounding) against central
    differences on `probes` random parameters."""
    rng = np.random.default_rng(seed)
    p = rng.standard_normal(N_PARAMS) * 0.3
    x = rng.standard_normal((n, N_IN))
    t = rng.standard_normal(n)
    _, g = loss_grad(p, x, t, rounding=False)
    worst = 0.0
    for i in rng.choice(N_PARAMS, probes, replace=False):
        q = p.copy()
        q[i] += eps
        lp, _ = loss_grad(q, x, t, rounding=False)
        q[i] -= 2 * eps
        lm, _ = loss_grad(q, x, t, rounding=False)
        fd = (lp - lm) / (2 * eps)
        worst = max(worst, abs(fd - g[i]) / max(abs(fd), 1e-8))
    return worst
