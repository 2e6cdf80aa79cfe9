"""Pins the autoencoder oracle (oracle/mlp_oracle.py): float64 gradients
against central finite differences of the loss, and its bfloat16 rounding
against torch's conversion."""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle  # noqa: E402


def _net(rng, n=16, k=3, ha=8, hb=6):
    ins = [n, ha, hb, k, hb, ha]
    outs = [ha, hb, k, hb, ha, n]
    Ws = [rng.normal(0, 0.4, (o, i)) for o, i in zip(outs, ins)]
    bs = [rng.normal(0, 0.1, o) for o in outs]
    return Ws, bs


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    Ws, bs = _net(rng)
    X = rng.normal(0, 1, (5, 16))
    loss, gW, gb = mlp_oracle.loss_and_gradients(Ws, bs, X, bf16=False)
    eps = 1e-6
    for l in range(6):
        for _ in range(4):
            i, j = rng.integers(Ws[l].shape[0]), rng.integers(Ws[l].shape[1])
            Wp = [w.copy() for w in Ws]
            Wm = [w.copy() for w in Ws]
            Wp[l][i, j] += eps
            Wm[l][i, j] -= eps
            fd = (mlp_oracle.loss_and_gradients(Wp, bs, X, False)[0] -
                  mlp_oracle.loss_and_gradients(Wm, bs, X, False)[0]) / (2 * eps)
            assert abs(fd - gW[l][i, j]) <= 1e-7 * max(1.0, abs(fd)), (l, i, j, fd, gW[l][i, j])
        i = rng.integers(bs[l].shape[0])
        bp = [b.copy() for b in bs]
        bm = [b.copy() for b in bs]
        bp[l][i] += eps
        bm[l][i] -= eps
        fd = (mlp_oracle.loss_and_gradients(Ws, bp, X, False)[0] -
              mlp_oracle.loss_and_gradients(Ws, bm, X, False)[0]) / (2 * eps)
        assert abs(fd - gb[l][i]) <= 1e-7 * max(1.0, abs(fd))


def test_bf16_rounding_matches_torch():
    import torch
    rng = np.random.default_rng(1)
    a = np.concatenate([rng.normal(0, 1, 10000), rng.normal(0, 1e-3, 1000), [0.0, -0.0, 1.0, 65504.0]])
    a = a.astype(np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(mlp_oracle.bf16_round(a), ref)
