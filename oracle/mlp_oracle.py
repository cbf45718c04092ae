"""Friction-surrogate network oracle -- TEST INFRASTRUCTURE ONLY.

float64 numpy forward and backward pass of the engine's 1-64-64-1 network
(SiLU hidden layers, softplus output = Cholesky factor L of the friction,
loss = mean (L - L*)^2), applying BF16 rounding exactly where the engine's
tensor-core kernels do: all parameters are used as BF16 values, hidden
layer 1 and the layer-2 error signal dz2 enter the BF16 GEMMs rounded.
Parameters are packed W1[64] b1[64] W2[64][64] (row = output unit) b2[64]
W3[64] b3[1].
"""
from __future__ import annotations

import numpy as np

NP = 4353
OFF = dict(W1=0, b1=64, W2=128, b2=128 + 4096, W3=4288, b3=4352)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, rounding=True):
    p = bf16(p) if rounding else np.asarray(p, np.float64)
    return (p[OFF["W1"]:OFF["W1"] + 64], p[OFF["b1"]:OFF["b1"] + 64], p[OFF["W2"]:OFF["W2"] + 4096].reshape(64, 64),
            p[OFF["b2"]:OFF["b2"] + 64], p[OFF["W3"]:OFF["W3"] + 64], p[OFF["b3"]])


def sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sig(z)


def dsilu(z):
    s = sig(z)
    return s * (1.0 + z * (1.0 - s))


def softplus(o):
    return np.where(o > 20.0, o, np.log1p(np.exp(np.minimum(o, 20.0))))


def forward(p, x, shift, scale, rounding=True):
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(p, rounding)
    u = (np.asarray(x, np.float32) - np.float32(shift)) * np.float32(scale)
    u = u.astype(np.float64)
    z1 = u[:, None] * W1[None, :] + b1[None, :]
    h1 = r(silu(z1))
    z2 = h1 @ W2.T + b2[None, :]
    o = silu(z2) @ W3 + b3
    return u, z1, h1, z2, o, softplus(o)


def predict_friction(p, x, shift, scale):
    return forward(p, x, shift, scale)[-1] ** 2


def loss_grad(p, x, t, shift, scale, rounding=True):
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(p, rounding)
    u, z1, h1, z2, o, L = forward(p, x, shift, scale, rounding)
    n = len(x)
    err = L - t
    loss = np.sum(err * err) / n
    dO = 2.0 * err / n * sig(o)
    g = np.zeros(NP)
    g[OFF["W3"]:OFF["W3"] + 64] = (dO[:, None] * silu(z2)).sum(0)
    g[OFF["b3"]] = dO.sum()
    dz2 = dO[:, None] * W3[None, :] * dsilu(z2)
    g[OFF["b2"]:OFF["b2"] + 64] = dz2.sum(0)
    dz2b = r(dz2)
    g[OFF["W2"]:OFF["W2"] + 4096] = (dz2b.T @ h1).reshape(-1)
    dh1 = dz2b @ W2
    dz1 = dh1 * dsilu(z1)
    g[OFF["W1"]:OFF["W1"] + 64] = (dz1 * u[:, None]).sum(0)
    g[OFF["b1"]:OFF["b1"] + 64] = dz1.sum(0)
    return loss, g
