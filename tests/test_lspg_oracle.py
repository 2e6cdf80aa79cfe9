"""Pins the LSPG oracle (oracle/lspg_oracle.py): every step it returns is a
stationary point of ||R(x)||^2 (the Gauss-Newton normal equations hold at the
returned latent) and equals the minimiser found by scipy's Levenberg-Marquardt
on the same BDF1 or BDF2 residual."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import lspg_oracle  # noqa: E402


def _setup(pda, oracle, n=16, frac=0.5, k=4, seed=0):
    full = pda.create_full_mesh((n, n), (-5, 5, -5, 5), 7, (False, False))
    rng = np.random.default_rng(seed)
    gids = np.sort(rng.choice(n * n, int(frac * n * n), replace=False))
    sm, st = pda.create_sample_mesh(full, gids)
    g, x, y, z, _, _ = sm._arrays()
    om = oracle.mesh_from_arrays(2, 7, g, x, y, z, (sm.dx(), sm.dy(), sm.dz()))
    po = oracle.problem(om, 3, 0, 2, 1, {"gravity": 7.0, "coriolis": -2.0, "pulseMagnitude": 0.15})
    s2st = np.searchsorted(st, gids)
    nst = len(st) * 3
    uref = np.zeros(nst)
    uref[0::3] = 1.0
    phi, _ = np.linalg.qr(rng.normal(0, 1, (nst, k)))
    phi *= 0.3
    return po, s2st, uref, phi, om


def test_lspg_oracle_steps_are_least_squares_minimisers(pda, oracle):
    from scipy.optimize import least_squares
    po, s2st, uref, phi, _ = _setup(pda, oracle)
    dec = lspg_oracle.affine_decoder(uref, phi)
    x0 = np.array([0.1, -0.05, 0.02, 0.0])
    dt = 0.01
    x1, traj = lspg_oracle.lspg_bdf1(po, s2st, dec, x0, dt, 1, iters=20, tol=1e-13)
    sd = lspg_oracle.sample_dofs(s2st, 3)
    yn = dec(x0)[0][sd]

    def resid(x):
        y, _ = dec(x)
        return -dt * po.velocity(y) + (y[sd] - yn)

    def jac(x):
        y, D = dec(x)
        _, rp, ci, jv = po.velocity_and_jacobian(y)
        J = sp.csr_matrix((jv, ci, rp), shape=(len(rp) - 1, len(y)))
        return -dt * (J @ D) + D[sd]

    R, JR = resid(x1), jac(x1)
    assert np.linalg.norm(JR.T @ R) <= 1e-9 * np.linalg.norm(JR) * max(np.linalg.norm(R), 1e-300)
    ref = least_squares(resid, x0, jac=jac, method="lm", xtol=1e-15, ftol=1e-15, gtol=1e-15)
    assert np.allclose(x1, ref.x, rtol=1e-8, atol=1e-11)


def test_lspg_oracle_bdf2_steps_are_least_squares_minimisers(pda, oracle):
    """BDF2 (Pressio's hyper-reduced policy: step 1 is BDF1, then
    R = -2/3 dt V(y) + (y - 4/3 y_n + 1/3 y_n-1))."""
    from scipy.optimize import least_squares
    po, s2st, uref, phi, _ = _setup(pda, oracle, seed=3)
    dec = lspg_oracle.affine_decoder(uref, phi)
    x0 = np.array([0.1, -0.05, 0.02, 0.03])
    dt = 0.01
    _, traj = lspg_oracle.lspg_bdf(po, s2st, dec, x0, dt, 3, order=2, iters=25, tol=1e-13)
    sd = lspg_oracle.sample_dofs(s2st, 3)
    # step 1 is the BDF1 step
    x1b, _ = lspg_oracle.lspg_bdf1(po, s2st, dec, x0, dt, 1, iters=25, tol=1e-13)
    assert np.array_equal(traj[0], x1b)
    for n in (1, 2):
        yn = dec(traj[n - 1])[0][sd]
        ynm1 = dec(traj[n - 2] if n >= 2 else x0)[0][sd]

        def resid(x):
            y, _ = dec(x)
            return -(2. / 3.) * dt * po.velocity(y) + (y[sd] - (4. / 3.) * yn + (1. / 3.) * ynm1)

        def jac(x):
            y, D = dec(x)
            _, rp, ci, jv = po.velocity_and_jacobian(y)
            J = sp.csr_matrix((jv, ci, rp), shape=(len(rp) - 1, len(y)))
            return -(2. / 3.) * dt * (J @ D) + D[sd]

        xs = traj[n]
        R, JR = resid(xs), jac(xs)
        assert np.linalg.norm(JR.T @ R) <= 1e-9 * np.linalg.norm(JR) * max(np.linalg.norm(R), 1e-300)
        ref = least_squares(resid, traj[n - 1], jac=jac, method="lm", xtol=1e-15, ftol=1e-15, gtol=1e-15)
        assert np.allclose(xs, ref.x, rtol=1e-8, atol=1e-11)


LSPG_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lspg")


def _lspg_gold_cases():
    return sorted(f[:-4] for f in os.listdir(LSPG_GOLD) if f.endswith(".npz"))


@pytest.mark.parametrize("name", _lspg_gold_cases())
def test_lspg_oracle_matches_pressio_golds(oracle, name):
    """The oracle's latent trajectories equal those of the reference's own
    hyper-reduced LSPG (vendored Pressio over the reference's slip-wall
    shallow-water problem on a reference-made sample mesh;
    tests/golden/make_lspg_golden.py), BDF1 and BDF2, with the same number of
    Gauss-Newton updates per step, to 1e-9 relative (the normal equations are
    solved by Householder QR there, by LU here)."""
    g = dict(np.load(os.path.join(LSPG_GOLD, name + ".npz")))
    gr, co, pu = (float(v) for v in g["params"])
    om = oracle.mesh_load(os.path.join(os.path.dirname(LSPG_GOLD), "meshes", "s2d_s7_20"))
    po = oracle.problem(om, 3, 0, 2, 1, {"gravity": gr, "coriolis": co, "pulseMagnitude": pu})
    dec = lspg_oracle.affine_decoder(g["uref"], g["phi"])
    _, traj = lspg_oracle.lspg_bdf(po, g["s2st"], dec, g["x0"], float(g["dt"]), int(g["steps"]), order=int(g["order"]),
                                   iters=int(g["updates"]), tol=0.0)
    traj = np.array(traj)
    scale = np.max(np.abs(g["traj"]))
    assert np.allclose(traj, g["traj"], rtol=1e-9, atol=1e-11 * scale), np.max(np.abs(traj - g["traj"])) / scale
