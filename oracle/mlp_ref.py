"""FP64 reference of the surrogate network's forward and backward pass -- TEST INFRASTRUCTURE ONLY.

Mirrors blackholerender_gb300/csrc/surrogate.cu: 3 -> 64 -> 64 -> 64 -> 2, SiLU, parameters in
the flat layout [W1 (64x3), b1, W2 (64x64), b2, W3 (64x64), b3, W4 (2x64), b4]. The loss of a
batch of n samples (x1, x2, sigma, y) with labels (0 escaped, 1 captured, 2 ignored) is
    L = sum_i [label_i == 0] (y_pred_i - y_i)^2 / n + w_c sum_i [label_i != 2] BCE(logit_i, label_i == 1) / n.
The GPU path rounds the hidden-layer weights and every activation (the output layer's inputs
too) to BF16; with quantize=True this reference does the same, everything else in FP64 (the
output layer's weights are FP32 on the GPU: three BF16 parts in inference).
"""
from __future__ import annotations

import numpy as np

H, IN, OUT = 64, 3, 2
OFF = {}
_o = 0
for name, size in (("W1", H * IN), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H), ("b3", H), ("W4", OUT * H),
                   ("b4", OUT)):
    OFF[name] = (_o, size)
    _o += size
NPARAMS = _o


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    d = {}
    for k, (o, n) in OFF.items():
        d[k] = p[o:o + n]
    d["W1"] = d["W1"].reshape(H, IN)
    d["W2"] = d["W2"].reshape(H, H)
    d["W3"] = d["W3"].reshape(H, H)
    d["W4"] = d["W4"].reshape(OUT, H)
    return d


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s + z * s * (1.0 - s)


def act(z, quantize=True):
    """The network's activation: SiLU, rounded to BF16 as on the GPU when quantize is set."""
    return bf16(silu(z)) if quantize else silu(z)


def forward(p, x, quantize=True):
    d = unpack(p)
    q = bf16 if quantize else (lambda a: np.asarray(a, dtype=np.float64))
    z1 = x @ d["W1"].T + d["b1"]
    h1 = act(z1, quantize)
    z2 = h1 @ q(d["W2"]).T + d["b2"]
    h2 = act(z2, quantize)
    z3 = h2 @ q(d["W3"]).T + d["b3"]
    h3 = act(z3, quantize)
    out = h3 @ d["W4"].T + d["b4"]
    return out, (z1, h1, z2, h2, z3, h3)


def loss_and_grad(p, samples, labels, w_c, quantize=True):
    """Returns (loss sums {sum err^2, sum BCE, n_y}, flat gradient of L)."""
    samples = np.asarray(samples, dtype=np.float64)
    labels = np.asarray(labels)
    n = len(samples)
    x, y = samples[:, :3], samples[:, 3]
    d = unpack(p)
    q = bf16 if quantize else (lambda a: np.asarray(a, dtype=np.float64))
    out, (z1, h1, z2, h2, z3, h3) = forward(p, x, quantize)
    my = labels == 0
    mc = labels != 2
    tgt = (labels == 1).astype(np.float64)
    err = out[:, 0] - y
    pr = 1.0 / (1.0 + np.exp(-out[:, 1]))
    dout = np.zeros_like(out)
    dout[:, 0] = np.where(my, 2.0 * err / n, 0.0)
    dout[:, 1] = np.where(mc, w_c * (pr - tgt) / n, 0.0)
    bce = np.maximum(out[:, 1], 0) - out[:, 1] * tgt + np.log1p(np.exp(-np.abs(out[:, 1])))
    sums = np.array([np.sum(err[my] ** 2), np.sum(bce[mc]), float(my.sum())])
    g = {}
    g["W4"] = dout.T @ h3
    g["b4"] = dout.sum(0)
    dz3 = (dout @ d["W4"]) * silu_grad(z3)
    g["W3"] = dz3.T @ h2
    g["b3"] = dz3.sum(0)
    dz2 = (dz3 @ q(d["W3"])) * silu_grad(z2)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ q(d["W2"])) * silu_grad(z1)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    flat = np.zeros(NPARAMS)
    for k, (o, sz) in OFF.items():
        flat[o:o + sz] = g[k].ravel()
    return sums, flat
