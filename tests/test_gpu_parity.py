"""GPU parity: the CUDA path through the C ABI against the reference.

* golden cases (tests/golden/cases, produced by the reference itself):
  velocity on the initial condition and on a seeded noisy state, within
  1e-13 relative per cell (floor 1e-3 x field max, the reference velocity is
  exactly zero in uniform regions); CSR row pointers and column indices
  bit-exact; Jacobian values within 1e-12 (same floor rule per row);
* the reference tests' own trajectory golds (Sod RK4, Riemann SSP-RK3,
  shallow-water RK4) through the device steppers;
* full-size, size-independent properties: sample-mesh rows equal full-mesh
  rows, periodic translation invariance, determinism.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, create_case_problem, golden_case, j_close, mesh_dir, v_close

pytestmark = pytest.mark.gpu

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
TRAJ = json.load(open(os.path.join(GOLDEN, "gold", "trajectories.json")))


def oracle_mod():
    import sys
    sys.path.insert(0, os.path.join(GOLDEN, "..", "..", "oracle"))
    import oracle_py
    return oracle_py


def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return torch


def problem_enum(pda, family, problem):
    return [pda.Euler1d, pda.Euler2d, pda.Euler3d, pda.Swe2d][family](problem)


def make_problem(pda, m, mesh=None):
    mesh = mesh or pda.load_cellcentered_uniform_mesh(mesh_dir(m["mesh"]))
    return mesh, create_case_problem(pda, m, mesh)


@pytest.mark.parametrize("case", sorted(MANIFEST))
def test_velocity_matches_reference(pda, case):
    torch = _torch()
    m = MANIFEST[case]
    g = golden_case(case)
    mesh, p = make_problem(pda, m)
    assert p.totalDofSampleMesh() == m["dofs_sample"]
    assert p.totalDofStencilMesh() == m["dofs_stencil"]
    # initial condition (host formulas, reference order): bit-exact
    u0 = p.initialCondition()
    assert np.array_equal(u0.cpu().numpy(), g["U0"])
    t = m.get("t", 0.0)
    for uk, vk in (("U0", "V0"), ("U1", "V1")):
        U = torch.from_numpy(g[uk]).cuda()
        V = p.createVelocity()
        p.velocity(U, t, V)
        v = V.cpu().numpy()
        ok, worst = v_close(v, g[vk], m["ndpc"])
        assert ok, f"{case} {vk}: worst relative error {worst:.3e}"
        if m["family"] != 3:
            # Euler velocities follow the reference's operation order exactly
            # (the shallow-water flux takes sqrt for glibc's pow(h, 0.5))
            assert np.array_equal(v, g[vk], equal_nan=True), f"{case} {vk}: not bit-identical"



@pytest.mark.parametrize("case", sorted(MANIFEST))
def test_jacobian_matches_reference(pda, case):
    torch = _torch()
    m = MANIFEST[case]
    g = golden_case(case)
    mesh, p = make_problem(pda, m)
    J = p.createJacobian()
    assert np.array_equal(J.rowptr.cpu().numpy(), g["rowptr"])
    assert np.array_equal(J.colidx.cpu().numpy(), g["colidx"])
    U = torch.from_numpy(g["U1"]).cuda()
    V = p.createVelocity()
    t = m.get("t", 0.0)
    p.rightHandSideAndJacobian(U, t, V, J)
    ok, worst = v_close(V.cpu().numpy(), g["Vj"], m["ndpc"])
    assert ok, f"{case} V (V+J path): worst {worst:.3e}"
    # J within 1e-12 of the row scale: the WENO weight derivatives cancel
    # terms far larger than the entries, and the reference's own x^3 (glibc
    # pow, not always correctly rounded) moves entries by up to ~1e-13 of it
    jv = J.values.cpu().numpy()
    ok, worst = j_close(jv, g["jvals"], g["rowptr"], rtol=m.get("jtol", 1e-12), floor_frac=1.0)
    assert ok, f"{case} J: worst {worst:.3e}"
    # ... and bit for bit equal to the oracle evaluated with a correctly
    # rounded x^3, the library's documented arithmetic
    orc = oracle_mod().load()
    orc.set_cube_mode(1)
    try:
        op = orc.problem(orc.mesh_load(mesh_dir(m["mesh"])), m["family"], m["problem"], m["scheme"], m["icflag"],
                         m.get("params"))
        Vo, _, _, jo = op.velocity_and_jacobian(g["U1"], t)
    finally:
        orc.set_cube_mode(0)
    if m["family"] != 3:
        assert np.array_equal(jv, jo, equal_nan=True), \
            f"{case}: J differs from the oracle ({np.sum(jv != jo)} entries)"
        assert np.array_equal(V.cpu().numpy(), Vo, equal_nan=True)
    else:
        ok, worst = j_close(jv, jo, g["rowptr"], rtol=1e-13, floor_frac=1.0)
        assert ok, f"{case}: J vs oracle worst {worst:.3e}"
    # jacobian() alone gives the same values
    J2 = p.createJacobian()
    p.jacobian(U, t, J2)
    assert torch.equal(torch.nan_to_num(J.values), torch.nan_to_num(J2.values))


@pytest.mark.parametrize("name", sorted(TRAJ))
def test_trajectory_gold(pda, name):
    """The reference tests' stored final states, reproduced by the device steppers."""
    t = TRAJ[name]
    mesh, p = make_problem(pda, t)
    U = p.initialCondition()
    for use_graph in (False, True):
        U = p.initialCondition()
        if t["stepper"] == "rk4":
            p.advance_rk4(U, 0.0, t["dt"], t["steps"], use_graph=use_graph)
        else:
            p.advance_ssprk3(U, 0.0, t["dt"], t["steps"], use_graph=use_graph)
        D = U.cpu().numpy()
        if name.startswith("sod"):
            gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
            assert np.allclose(D, gold, rtol=t["rtol"], atol=t["atol"])
        elif name.startswith("riemann"):
            gold = np.load(os.path.join(GOLDEN, "gold", name + ".npz"))
            D = D.reshape(-1, 4)
            rho = D[:, 0]
            u, v = D[:, 1] / rho, D[:, 2] / rho
            pr = ((5. + 2.) / 5. - 1.) * (D[:, 3] - rho * (u ** 2 + v ** 2) * 0.5)
            assert np.allclose(rho, gold["rho"], rtol=t["rtol"], atol=t["atol"])
            assert np.allclose(pr, gold["p"], rtol=t["rtol"], atol=t["atol"])
        elif name.startswith(("cross", "dmr")):
            gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
            assert np.allclose(D.reshape(-1, 4)[:, 0], gold, rtol=t["rtol"], atol=t["atol"])
        else:
            gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
            assert np.allclose(D.reshape(-1, 3)[:, 0], gold, rtol=t["rtol"], atol=t["atol"])


GENTRAJ = json.load(open(os.path.join(GOLDEN, "gold", "trajectories_generated_mesh.json")))


@pytest.mark.parametrize("name", sorted(GENTRAJ))
def test_generated_mesh_trajectory_gold(pda, name):
    """Golds of the reference tests whose meshes the library generates here:
    the Python tests (cross shock 80x40, 1000 steps; double Mach reflection
    200x50, 500 steps, first order and WENO3) and the 3D Sedov symmetry runs
    (20^3 and 20x25x28, first order and WENO3, 250 steps, whole state), all
    advanced by the device SSP-RK3.  The device stepper applies Pressio's
    update order and the Python driver its own: both are the same scheme and
    the gold's own tolerance holds."""
    t = GENTRAJ[name]
    mesh = pda.create_full_mesh(tuple(t["n"]), tuple(t["bounds"]), t["stencil"])
    enum = (pda.Euler2d if t["family"] == 1 else pda.Euler3d)(t["problem"])
    p = pda.create_problem(mesh, enum, pda.InviscidFluxReconstruction(t["scheme"]), t["icflag"])
    U = p.initialCondition()
    p.advance_ssprk3(U, 0.0, t["dt"], t["steps"])
    D = U.cpu().numpy()
    got = D.reshape(-1, p.numDofPerCell())[:, 0] if t["field"] == "rho" else D
    gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
    assert np.allclose(got, gold, rtol=t["rtol"], atol=t["atol"])


def test_apply_jacobian_matches_spmv(pda):
    torch = _torch()
    m = MANIFEST["riemann_w5"]
    g = golden_case("riemann_w5")
    mesh, p = make_problem(pda, m)
    U = torch.from_numpy(g["U1"]).cuda()
    rng = np.random.default_rng(7)
    B = rng.standard_normal((m["dofs_stencil"], 3))
    import scipy.sparse as sp
    Jref = sp.csr_matrix((g["jvals"], g["colidx"], g["rowptr"]), shape=(m["dofs_sample"], m["dofs_stencil"]))
    R = torch.empty((m["dofs_sample"], 3), dtype=torch.float64, device="cuda")
    p.applyJacobian(U, torch.from_numpy(B).cuda(), 0.0, R)
    np.testing.assert_allclose(R.cpu().numpy(), Jref @ B, rtol=1e-11, atol=1e-9)
    r1 = torch.empty(m["dofs_sample"], dtype=torch.float64, device="cuda")
    p.applyJacobian(U, torch.from_numpy(B[:, 0].copy()).cuda(), 0.0, r1)
    np.testing.assert_allclose(r1.cpu().numpy(), Jref @ B[:, 0], rtol=1e-11, atol=1e-9)


def test_host_buffer_entry_points(pda):
    """pda_velocity_host / pda_velocity_and_jacobian_host (the plugin call a
    caller holding host vectors makes) equal the device entry points."""
    torch = _torch()
    m = MANIFEST["swe_w5"]
    g = golden_case("swe_w5")
    mesh, p = make_problem(pda, m)
    Vh = np.empty(m["dofs_sample"])
    p.velocity_host(np.ascontiguousarray(g["U1"]), 0.0, Vh)
    V = p.createVelocity()
    p.velocity(torch.from_numpy(g["U1"]).cuda(), 0.0, V)
    assert np.array_equal(Vh, V.cpu().numpy())
    ok, _ = v_close(Vh, g["V1"], 3)
    assert ok


@pytest.mark.parametrize("shape,family,problem,scheme,ic,per", [
    ((515, 203), "Euler2d", 4, 2, 2, False),   # Neumann mirror, uneven sides
    ((96, 96), "Swe2d", 0, 1, 1, False),       # slip wall, WENO3
    ((130, 100), "Euler2d", 0, 2, 1, True),    # periodic
    ((100, 112), "Euler2d", 4, 0, 2, False),   # first order
    ((90, 60), "Euler2d", 4, 2, 2, False),     # below the banded path's 96 rows
    ((40, 36, 50), "Euler3d", 0, 2, 1, True),  # periodic
])
def test_host_buffer_velocity_equals_device_full_meshes(pda, shape, family, problem, scheme, ic, per):
    """The host-buffer velocity (the C-ABI call with host vectors) on full
    structured meshes equals the device path bit for bit, call after call
    (2D meshes of at least 96 rows: six row bands on their own streams, copies
    overlapping the other band's kernels)."""
    torch = _torch()
    dim = len(shape)
    bounds = (-1.0, 1.0) * dim if dim == 3 else (0.0, 1.0, 0.0, 1.0)
    mesh = pda.create_full_mesh(shape, bounds, 7, (per,) * dim)
    p = pda.create_problem(mesh, getattr(pda, family)(problem), pda.InviscidFluxReconstruction(scheme), ic)
    U = p.initialCondition()
    gen = torch.Generator(device="cuda").manual_seed(3)
    U += (torch.rand(U.shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1) * 1e-3
    V = p.createVelocity()
    p.velocity(U, 0.0, V)
    Vh = np.empty(p.totalDofSampleMesh())
    for _ in range(2):
        p.velocity_host(np.ascontiguousarray(U.cpu().numpy()), 0.0, Vh)
        assert np.array_equal(Vh, V.cpu().numpy())


# ------------------------------------------------------- full-size properties

def _riemann_full(pda, n, scheme=2, noise_seed=None):
    torch = _torch()
    mesh = pda.create_full_mesh((n, n), (0.0, 1.0, 0.0, 1.0), 7)
    p = pda.create_problem(mesh, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction(scheme), 2)
    U = p.initialCondition()
    if noise_seed is not None:
        gen = torch.Generator(device="cuda").manual_seed(noise_seed)
        U += (torch.rand(U.shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1) * 1e-3
    return mesh, p, U


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_sample_mesh_rows_equal_full_mesh_rows_1024(pda, scheme):
    """Reference sample-mesh consistency (tests_cpp/eigen_2d_euler_sample_mesh_test1):
    V on a sample mesh equals the full-mesh V at the sampled cells.  At 1024^2
    the full mesh takes the structured face-once kernels and the sample mesh
    the per-row kernels, so this checks one against the other at full size."""
    torch = _torch()
    mesh, p, U = _riemann_full(pda, 1024, scheme, noise_seed=11)
    V = p.createVelocity()
    p.velocity(U, 0.0, V)
    assert torch.isfinite(V).all()
    rng = np.random.default_rng(5)
    n = 1024 * 1024
    gids = np.unique(np.concatenate([rng.choice(n, 3000, replace=False),
                                     np.arange(0, 1024 * 4), np.arange(n - 1024 * 4, n),
                                     np.arange(0, n, 1024), np.arange(1023, n, 1024)]))
    sm, stencil_gids = pda.create_sample_mesh(mesh, gids)
    ps = pda.create_problem(sm, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction(scheme), 2)
    Us = U.view(-1, 4)[torch.from_numpy(stencil_gids).cuda()].reshape(-1).contiguous()
    Vs = ps.createVelocity()
    ps.velocity(Us, 0.0, Vs)
    ref = V.view(-1, 4)[torch.from_numpy(gids).cuda()].reshape(-1)
    assert torch.equal(Vs, ref)


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_sample_mesh_rows_equal_full_mesh_faces_1d(pda, scheme):
    """1D full meshes below 8192 cells take the per-row kernel for every row
    (the face pass would leave most SMs idle); at 20,000 cells the Sod mesh
    takes the structured face pass, so its velocity at sampled cells must
    equal the sample mesh's (per-row kernel) bit for bit, boundary rows
    included."""
    torch = _torch()
    n = 20000
    mesh = pda.create_full_mesh((n,), (-0.5, 0.5), 7, (False,))
    p = pda.create_problem(mesh, pda.Euler1d.Sod, pda.InviscidFluxReconstruction(scheme))
    U = p.initialCondition()
    gen = torch.Generator(device="cuda").manual_seed(17)
    U += (torch.rand(U.shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1) * 1e-3
    V = p.createVelocity()
    p.velocity(U, 0.0, V)
    assert torch.isfinite(V).all()
    rng = np.random.default_rng(9)
    gids = np.unique(np.concatenate([rng.choice(n, 500, replace=False), np.arange(0, 8), np.arange(n - 8, n),
                                     np.arange(n // 2 - 4, n // 2 + 4)]))
    sm, stencil_gids = pda.create_sample_mesh(mesh, gids)
    ps = pda.create_problem(sm, pda.Euler1d.Sod, pda.InviscidFluxReconstruction(scheme))
    Us = U.view(-1, 3)[torch.from_numpy(stencil_gids).cuda()].reshape(-1).contiguous()
    Vs = ps.createVelocity()
    ps.velocity(Us, 0.0, Vs)
    ref = V.view(-1, 3)[torch.from_numpy(gids).cuda()].reshape(-1)
    assert torch.equal(Vs, ref)


def test_periodic_translation_invariance_512(pda):
    torch = _torch()
    mesh = pda.create_full_mesh((512, 512), (-1.0, 1.0, -1.0, 1.0), 7, (True, True))
    p = pda.create_problem(mesh, pda.Euler2d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5)
    gen = torch.Generator(device="cuda").manual_seed(3)
    U = p.initialCondition()
    U += (torch.rand(U.shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1) * 1e-2
    V = p.createVelocity()
    p.velocity(U, 0.0, V)
    Ur = U.view(512, 512, 4).roll(shifts=(5, -7), dims=(0, 1)).reshape(-1).contiguous()
    Vr = p.createVelocity()
    p.velocity(Ur, 0.0, Vr)
    assert torch.equal(Vr, V.view(512, 512, 4).roll(shifts=(5, -7), dims=(0, 1)).reshape(-1))


def test_determinism_and_jacobian_sample_consistency_256(pda):
    torch = _torch()
    mesh, p, U = _riemann_full(pda, 256, 2, noise_seed=2)
    J = p.createJacobian()
    V = p.createVelocity()
    p.rightHandSideAndJacobian(U, 0.0, V, J)
    V2 = p.createVelocity()
    J2 = p.createJacobian()
    p.rightHandSideAndJacobian(U, 0.0, V2, J2)
    assert torch.equal(V, V2) and torch.equal(J.values, J2.values)
    assert torch.isfinite(J.values).all()
    # sample mesh rows/columns of J equal the full-mesh entries
    rng = np.random.default_rng(9)
    gids = np.unique(np.concatenate([rng.choice(256 * 256, 400, replace=False), np.arange(0, 600)]))
    sm, st = pda.create_sample_mesh(mesh, gids)
    ps = pda.create_problem(sm, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2)
    Js = ps.createJacobian()
    Us = U.view(-1, 4)[torch.from_numpy(st).cuda()].reshape(-1).contiguous()
    Vs = ps.createVelocity()
    ps.rightHandSideAndJacobian(Us, 0.0, Vs, Js)
    Jf = J.to_scipy()
    Jsm = Js.to_scipy()
    rows_full = (gids[:, None] * 4 + np.arange(4)[None, :]).reshape(-1)
    cols_full = (st[:, None] * 4 + np.arange(4)[None, :]).reshape(-1)
    sub = Jf[rows_full][:, cols_full].toarray()
    assert np.array_equal(sub, Jsm.toarray())
    assert torch.equal(Vs, V.view(-1, 4)[torch.from_numpy(gids).cuda()].reshape(-1))


def test_sedov3d_weno5_refused_as_in_the_reference(pda):
    """The reference's 3D Sedov ghost filler has no WENO5 layers and throws
    at evaluation; the library refuses the evaluation the same way."""
    torch = _torch()
    mesh = pda.create_full_mesh((8, 8, 8), (0.0, 0.4, 0.0, 0.4, 0.0, 0.4), 7)
    p = pda.create_problem(mesh, pda.Euler3d.SedovSymmetry, pda.InviscidFluxReconstruction.Weno5)
    U = p.initialCondition()
    V = p.createVelocity()
    with pytest.raises(pda.PdaError):
        p.velocity(U, 0.0, V)
    torch.cuda.synchronize()


def test_host_buffer_velocity_graph_replay_pinned(pda):
    """Repeated host-buffer calls with the same pinned buffers and time replay
    one captured CUDA graph from the second call on.  Each replay still copies
    the buffers' current contents, and a call with another output buffer or
    another time takes the direct path again; every result equals the device
    velocity bit for bit."""
    torch = _torch()
    mesh = pda.create_full_mesh((128, 96), (0.0, 1.0, 0.0, 1.0), 7)
    p = pda.create_problem(mesh, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2)
    U0 = p.initialCondition()
    n = p.totalDofSampleMesh()
    Uh = torch.empty(U0.numel(), dtype=torch.float64).pin_memory()
    Vh = torch.empty(n, dtype=torch.float64).pin_memory()
    Vh2 = torch.empty(n, dtype=torch.float64).pin_memory()
    gen = torch.Generator(device="cuda").manual_seed(5)
    V = p.createVelocity()
    for k, (out, t) in enumerate([(Vh, 0.0), (Vh, 0.0), (Vh, 0.0), (Vh2, 0.0), (Vh, 0.5), (Vh, 0.5), (Vh, 0.5)]):
        U = U0 + (torch.rand(U0.shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1) * 1e-3
        Uh.copy_(U.cpu())
        p.velocity_host(Uh.numpy(), t, out.numpy())
        p.velocity(U, t, V)
        assert torch.equal(out, V.cpu()), k
