"""pda_velocity_noalloc: the allocation-free velocity entry point.

It runs the same face and balance kernels as pda_velocity with the face-flux
scratch in the library's static device array, so its output must equal
pda_velocity's bit for bit.  Each case calls it twice in a row on different
states (the second call must not see anything left over from the first) and
checks that device free memory does not move across those calls.  The file
is collected last so that it also runs after every other GPU test."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

PDA_ERR_INVALID_ARGUMENT = -1
PDA_ERR_UNSUPPORTED = -4


def _noalloc(pda):
    L = pda.lib()
    f = L.pda_velocity_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    return f


def _call(pda, prob, U, V):
    return _noalloc(pda)(prob._h, C.c_void_p(U.data_ptr()), 0.0, C.c_void_p(V.data_ptr()))


def _states(prob, seed):
    import torch
    U0 = prob.initialCondition()
    g = torch.Generator(device="cuda").manual_seed(seed)
    noise = lambda: (torch.rand(U0.shape, generator=g, device="cuda", dtype=torch.float64) - 0.5) * 2e-3
    return U0 + noise(), U0 + noise()


def _check_two_calls(pda, prob, seed):
    import torch
    U1, U2 = _states(prob, seed)
    R1, R2 = prob.createVelocity(), prob.createVelocity()
    prob.velocity(U1, 0.0, R1)
    prob.velocity(U2, 0.0, R2)
    V1, V2 = prob.createVelocity(), prob.createVelocity()
    V1.fill_(np.nan)
    V2.fill_(np.nan)
    # first call per device: symbol lookup (may load the module holding the array)
    W = prob.createVelocity()
    assert _call(pda, prob, U1, W) == 0, pda.lib().pda_last_error().decode()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert _call(pda, prob, U1, V1) == 0, pda.lib().pda_last_error().decode()
    assert _call(pda, prob, U2, V2) == 0, pda.lib().pda_last_error().decode()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    assert torch.equal(V1, R1)
    assert torch.equal(V2, R2)
    assert torch.equal(W, R1)


def _mesh2d(pda, n, periodic=False):
    return pda.create_full_mesh((n, n), (-1, 1, -1, 1) if periodic else (0, 1, 0, 1), 7,
                                (periodic, periodic))


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_noalloc_euler2d_riemann_matches_velocity(pda, scheme):
    m = _mesh2d(pda, 256)
    p = pda.create_problem(m, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction(scheme), 2)
    _check_two_calls(pda, p, 20 + scheme)


@pytest.mark.gpu
def test_noalloc_euler3d_periodic_matches_velocity(pda):
    n = 48
    m = pda.create_full_mesh((n, n, n), (-1, 1, -1, 1, -1, 1), 7, (True, True, True))
    p = pda.create_problem(m, pda.Euler3d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5)
    _check_two_calls(pda, p, 31)


@pytest.mark.gpu
def test_noalloc_swe_slip_wall_matches_velocity(pda):
    m = pda.create_full_mesh((128, 128), (-5, 5, -5, 5), 7, (False, False))
    p = pda.create_problem(m, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5)
    _check_two_calls(pda, p, 41)


@pytest.mark.gpu
def test_noalloc_near_boundary_rows_after_first_velocity(pda):
    """Sod (1D, near-boundary rows): refused until pda_velocity has uploaded
    the row table, then identical to pda_velocity."""
    import torch
    m = pda.create_full_mesh((2000,), (-0.5, 0.5), 7, (False,))
    p = pda.create_problem(m, pda.Euler1d.Sod, pda.InviscidFluxReconstruction.Weno5)
    U = p.initialCondition()
    V = p.createVelocity()
    assert _call(pda, p, U, V) == PDA_ERR_UNSUPPORTED
    assert "pda_velocity" in pda.lib().pda_last_error().decode()
    R = p.createVelocity()
    p.velocity(U, 0.0, R)
    torch.cuda.synchronize()
    _check_two_calls(pda, p, 51)


@pytest.mark.gpu
def test_noalloc_rejects_mesh_beyond_static_limit(pda):
    m = _mesh2d(pda, 1024)
    p = pda.create_problem(m, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2)
    U = p.initialCondition()
    V = p.createVelocity()
    assert _call(pda, p, U, V) == PDA_ERR_INVALID_ARGUMENT
    msg = pda.lib().pda_last_error().decode()
    assert "static limit" in msg and str(2 * 1025 * 1024 * 4) in msg


@pytest.mark.gpu
def test_noalloc_rejects_sample_mesh(pda):
    full = _mesh2d(pda, 32)
    sm, _ = pda.create_sample_mesh(full, np.arange(0, 32 * 32, 7))
    p = pda.create_problem(sm, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2)
    import torch
    U = torch.zeros(p.totalDofStencilMesh(), dtype=torch.float64, device="cuda")
    V = p.createVelocity()
    assert _call(pda, p, U, V) == PDA_ERR_UNSUPPORTED
