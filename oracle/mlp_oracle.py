"""TEST INFRASTRUCTURE ONLY — FP64 numpy restatement of the engine's size
model (sparqsim_gb300/csrc/predictor.cu): a 48 -> 64 -> 64 -> 2 ReLU MLP,
mean-squared-error loss over all outputs, its gradient by backpropagation,
and the Adam update (Kingma & Ba 2015, beta1 0.9, beta2 0.999, eps 1e-8).
The reference has no such model; this is the checker of the GPU kernels'
forward, backward and update. Parameter layout: W1[48][64], b1, W2[64][64],
b2, W3[64][2], b3, flattened in that order."""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 48, 64, 2
SHAPES = [("W1", (IN, HID)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (HID, OUT)), ("b3", (OUT,))]
PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def forward(p, x):
    w = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"] + w["b1"]
    a1 = np.maximum(z1, 0.0)
    z2 = a1 @ w["W2"] + w["b2"]
    a2 = np.maximum(z2, 0.0)
    y = a2 @ w["W3"] + w["b3"]
    return y, (x, z1, a1, z2, a2)


def loss_and_grad(p, x, t):
    w = unpack(p)
    y, (x, z1, a1, z2, a2) = forward(p, x)
    t = np.asarray(t, dtype=np.float64)
    m = y.size
    loss = float(np.sum((y - t) ** 2) / m)
    dy = 2.0 * (y - t) / m
    g = {"W3": a2.T @ dy, "b3": dy.sum(axis=0)}
    d2 = (dy @ w["W3"].T) * (z2 > 0)
    g["W2"], g["b2"] = a1.T @ d2, d2.sum(axis=0)
    d1 = (d2 @ w["W2"].T) * (z1 > 0)
    g["W1"], g["b1"] = x.T @ d1, d1.sum(axis=0)
    return loss, pack(g)


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update; step counts from 1."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
