"""Test infrastructure only (the oracle): numpy restatement of the autoencoder
forward / backward pass of the library (csrc/ae.cu), used to check its
gradients.  Imported by tests/ only.

With ``bf16=True`` it rounds where the device rounds (bf16 weight copies,
bf16 activations between layers, bf16 output gradient and bf16 dA), and
accumulates in float64; with ``bf16=False`` everything is float64 and the
gradients are exact derivatives of the loss (pinned by finite differences in
tests/test_mlp_oracle.py).

Network (padded shapes as on the device): layers 0..5 with
W_l [out x in], b_l [out]; ELU after layers 0, 1, 3, 4; loss = mean over all
entries of (Y - X)^2.
"""
from __future__ import annotations

import numpy as np

ELU_LAYERS = (True, True, False, True, True, False)


def bf16_round(a):
    """Round float values to bfloat16 (nearest, ties to even) and return float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def elu(a):
    return np.where(a > 0, a, np.expm1(np.minimum(a, 0)))


def delu(a):
    return np.where(a > 0, 1.0, np.exp(np.minimum(a, 0)))


def forward(Ws, bs, X, bf16=True):
    r = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    Wb = [r(W) for W in Ws]
    h = r(X)
    pres, hins = [], []
    for l in range(6):
        hins.append(h)
        pre = h @ Wb[l].T + bs[l]
        if bf16:
            pre = pre.astype(np.float32).astype(np.float64)
        pres.append(pre)
        if l < 5:
            h = r(elu(pre)) if ELU_LAYERS[l] else r(pre)
    return pres[5], pres, hins, Wb


def loss_and_gradients(Ws, bs, X, bf16=True):
    """Returns (loss, [gW_l], [gb_l])."""
    r = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    Y, pres, hins, Wb = forward(Ws, bs, X, bf16)
    Xr = r(X)
    total = Y.size
    d = Y - Xr
    loss = float(np.sum(d * d) / total)
    dA = r((2.0 / total) * d)
    gW, gb = [None] * 6, [None] * 6
    for l in range(5, -1, -1):
        gW[l] = dA.T @ hins[l]
        gb[l] = dA.sum(axis=0)
        if l == 0:
            break
        dH = dA @ Wb[l]
        dA = r(dH * delu(pres[l - 1])) if ELU_LAYERS[l - 1] else r(dH)
    return loss, gW, gb
