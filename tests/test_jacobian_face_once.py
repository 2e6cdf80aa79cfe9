"""The face-once Jacobian (k_jfaces + k_jassemble on natural-order full
meshes) against the per-row formulation (k_rows_vj_inner), which the oracle
and the reference tests pin bit for bit.

A sample mesh made of every cell but one is not a full mesh, so its rows go
through the per-row kernels; its V and J rows must equal the full-mesh rows
bit for bit for every family the face-once path serves."""
from __future__ import annotations

import numpy as np
import pytest

CASES = [
    # id, family enum attr, problem, n, bounds, periodic, scheme, icflag
    ("euler2d_smooth_periodic_w5", "Euler2d", "PeriodicSmooth", (40, 40), (-1, 1, -1, 1), (True, True), 2, 1),
    ("euler2d_smooth_periodic_w3", "Euler2d", "PeriodicSmooth", (40, 40), (-1, 1, -1, 1), (True, True), 1, 1),
    ("euler2d_riemann_w5", "Euler2d", "Riemann", (48, 40), (0, 1, 0, 1), (False, False), 2, 2),
    ("euler2d_riemann_w3", "Euler2d", "Riemann", (48, 40), (0, 1, 0, 1), (False, False), 1, 2),
    ("swe_slipwall_w5", "Swe2d", "SlipWall", (40, 44), (-5, 5, -5, 5), (False, False), 2, 1),
    ("euler1d_sod_w5", "Euler1d", "Sod", (300,), (-0.5, 0.5), (False,), 2, 1),
    ("euler3d_periodic_w3", "Euler3d", "PeriodicSmooth", (12, 10, 9), (-1, 1, -1, 1, -1, 1), (True, True, True),
     1, 1),
    ("euler3d_periodic_w5", "Euler3d", "PeriodicSmooth", (12, 10, 9), (-1, 1, -1, 1, -1, 1), (True, True, True),
     2, 1),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_face_once_jacobian_equals_per_row(pda, case):
    import torch
    _, fam, prob, n, bounds, periodic, scheme, ic = case
    stencil = 7 if (scheme == 2 or len(n) < 3) else 5
    mesh = pda.create_full_mesh(n, bounds, stencil, periodic)
    enum = getattr(getattr(pda, fam), prob)
    p = pda.create_problem(mesh, enum, pda.InviscidFluxReconstruction(scheme), ic)
    ndpc = p.numDofPerCell()
    U = p.initialCondition()
    g = torch.Generator(device="cuda").manual_seed(7)
    U += (torch.rand(U.shape, generator=g, device="cuda", dtype=torch.float64) - 0.5) * 2e-3
    J = p.createJacobian()
    V = p.createVelocity()
    p.rightHandSideAndJacobian(U, 0.0, V, J)
    ncell = int(np.prod(n))
    gids = np.setdiff1d(np.arange(ncell), [ncell // 2 + 3])
    sm, st = pda.create_sample_mesh(mesh, gids)
    ps = pda.create_problem(sm, enum, pda.InviscidFluxReconstruction(scheme), ic)
    Us = U.view(-1, ndpc)[torch.from_numpy(st).cuda()].reshape(-1).contiguous()
    Js = ps.createJacobian()
    Vs = ps.createVelocity()
    ps.rightHandSideAndJacobian(Us, 0.0, Vs, Js)
    assert torch.equal(Vs, V.view(-1, ndpc)[torch.from_numpy(gids).cuda()].reshape(-1))
    rows = (gids[:, None] * ndpc + np.arange(ndpc)[None, :]).reshape(-1)
    cols = (st[:, None] * ndpc + np.arange(ndpc)[None, :]).reshape(-1)
    sub = J.to_scipy()[rows][:, cols].tocsr()
    sub.sort_indices()
    js = Js.to_scipy().tocsr()
    js.sort_indices()
    assert np.array_equal(sub.indptr, js.indptr) and np.array_equal(sub.indices, js.indices)
    assert np.array_equal(sub.data, js.data)
