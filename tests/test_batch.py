"""Batched problems (one launch per residual phase over all instances).

Every tile of the batched kernels runs the single-problem code on one
instance, so each instance's velocity and SSP-RK3 trajectory must equal the
single-problem entry points bit for bit, for every tile shape the autotuner
may pick; one small instance is also checked against the oracle."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
from conftest import v_close  # noqa: E402


def _swe_batch(pda, sizes, scheme, seed=3):
    rng = np.random.default_rng(seed)
    probs = []
    for n in sizes:
        m = pda.create_full_mesh((n, n), (-5, 5, -5, 5), 7, (False, False))
        params = {"gravity": rng.uniform(5, 10), "coriolis": rng.uniform(-4, -1),
                  "pulseMagnitude": rng.uniform(0.05, 0.2)}
        probs.append(pda.create_problem(m, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction(scheme), 1,
                                        params))
    return probs


def _noisy(batch, seed):
    import torch
    U = batch.initialCondition()
    g = torch.Generator(device="cuda").manual_seed(seed)
    return U + (torch.rand(U.shape, generator=g, device="cuda", dtype=torch.float64) - 0.5) * 2e-3


def _single_velocities(probs, batch, U):
    out = []
    for i, p in enumerate(probs):
        V = p.createVelocity()
        p.velocity(batch.instance(U, i).contiguous(), 0.0, V)
        out.append(V)
    return out


SIZES = [64, 96, 64, 128, 160, 7 * 11, 96]


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_batch_swe_velocity_bitwise_every_tile_shape(pda, scheme):
    import torch
    probs = _swe_batch(pda, SIZES, scheme)
    B = pda.create_batch(probs)
    U = _noisy(B, 11 + scheme)
    ref = _single_velocities(probs, B, U)
    for shape in range(B.num_tile_shapes()):
        for a in range(2):
            B.set_tile_shape(a, shape)
        V = torch.full_like(U, float("nan"))
        B.velocity(U, 0.0, V)
        for i in range(len(probs)):
            assert torch.equal(B.instance(V, i), ref[i]), (shape, i)


@pytest.mark.gpu
def test_batch_swe_autotune_then_ssprk3_matches_single_problems(pda):
    import torch
    probs = _swe_batch(pda, SIZES, 2, seed=5)
    B = pda.create_batch(probs)
    U = B.initialCondition()
    ms = B.autotune(U, reps=2)
    assert np.all(ms[:2, : B.num_tile_shapes()] > 0)
    Ug, Un = U.clone(), U.clone()
    B.advance_ssprk3(Ug, 0.0, 0.005, 12, use_graph=True)
    B.advance_ssprk3(Un, 0.0, 0.005, 12, use_graph=False)
    assert torch.equal(Ug, Un)
    for i, p in enumerate(probs):
        Ui = B.instance(U, i).clone()
        p.advance_ssprk3(Ui, 0.0, 0.005, 12)
        assert torch.equal(B.instance(Ug, i), Ui), i


@pytest.mark.gpu
def test_batch_swe_small_instance_matches_oracle(pda, oracle, tmp_path):
    probs = _swe_batch(pda, [64, 32], 2, seed=9)
    B = pda.create_batch(probs)
    U = B.initialCondition()
    B.advance_ssprk3(U, 0.0, 0.005, 6)
    m = pda.create_full_mesh((64, 64), (-5, 5, -5, 5), 7, (False, False))
    m.write(str(tmp_path / "m"))
    om = oracle.mesh_load(str(tmp_path / "m"))
    p0 = probs[0]
    params = {k: p0.queryParameter(k) for k in ("gravity", "coriolis", "pulseMagnitude")}
    po = oracle.problem(om, 3, 0, 2, 1, params)
    Uo = po.initial_condition()
    po.ssprk3(Uo, 0.0, 0.005, 6)
    ok, worst = v_close(B.instance(U, 0).cpu().numpy(), Uo, 3, rtol=1e-12)
    assert ok, worst


@pytest.mark.gpu
def test_batch_euler2d_and_euler3d_bitwise(pda):
    import torch
    probs = []
    for n in (48, 80, 33):
        m = pda.create_full_mesh((n, n), (0, 1, 0, 1), 7, (False, False))
        probs.append(pda.create_problem(m, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2))
    B = pda.create_batch(probs)
    U = _noisy(B, 21)
    ref = _single_velocities(probs, B, U)
    V = torch.zeros_like(U)
    B.velocity(U, 0.0, V)
    for i in range(len(probs)):
        assert torch.equal(B.instance(V, i), ref[i])
    probs3 = []
    for n in (16, 24):
        m = pda.create_full_mesh((n, n, n), (-1, 1, -1, 1, -1, 1), 7, (True, True, True))
        probs3.append(pda.create_problem(m, pda.Euler3d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5))
    B3 = pda.create_batch(probs3)
    assert B3.num_tile_shapes() == 1
    U3 = _noisy(B3, 22)
    ref3 = _single_velocities(probs3, B3, U3)
    V3 = torch.zeros_like(U3)
    B3.velocity(U3, 0.0, V3)
    for i in range(len(probs3)):
        assert torch.equal(B3.instance(V3, i), ref3[i])


@pytest.mark.gpu
def test_batch_rejects_mixed_or_unsupported_instances(pda):
    a = _swe_batch(pda, [32], 2)[0]
    b = _swe_batch(pda, [32], 1)[0]
    with pytest.raises(pda.PdaError):
        pda.create_batch([a, b])
    m = pda.create_full_mesh((200,), (-0.5, 0.5), 7, (False,))
    sod = pda.create_problem(m, pda.Euler1d.Sod, pda.InviscidFluxReconstruction.Weno5)
    with pytest.raises(pda.PdaError):
        pda.create_batch([sod])
