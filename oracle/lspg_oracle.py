"""Test infrastructure only (the oracle): numpy restatement of hyper-reduced
LSPG with BDF1 / BDF2 and Gauss-Newton, the algorithm of Pressio's
LspgUnsteadyResidualJacobianPolicyHypRed
(tests_cpp/pressio/include/pressio/rom/impl/lspg_unsteady_rj_policy_hypred.hpp:
100-264; constants from ode/ode_constants.hpp:57-73: BDF1 c_n = -1, c_f = -1;
BDF2 c_n = -4/3, c_nm1 = 1/3, c_f = -2/3, whose first step is a BDF1 step),
over the C oracle's sample-mesh velocity and Jacobian.  Imported by tests/
only.

Per step n -> n+1 and iteration, with y(x) the trial state on the stencil mesh
and D = dy/dx:
    R  = cf V(y) + (y + c_n y_n [+ c_nm1 y_nm1])|sample,   cf = c_f dt
    JR = cf Jf(y) D + D|sample
    (JR^T JR) dx = JR^T R,   x <- x - dx   (stop when |dx| < tol)
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def sample_dofs(s2st, ndpc):
    s2st = np.asarray(s2st, dtype=np.int64)
    return (s2st[:, None] * ndpc + np.arange(ndpc)[None, :]).reshape(-1)


def affine_decoder(uref, phi):
    def dec(x):
        return uref + phi @ x, phi
    return dec


def mlp_decoder(uref, scale, W1, b1, W2, b2, W3, b3):
    """y = uref + scale * (W3 elu(W2 elu(W1 x + b1) + b2) + b3) in float64."""
    def elu(a):
        return np.where(a > 0, a, np.expm1(np.minimum(a, 0)))

    def delu(a):
        return np.where(a > 0, 1.0, np.exp(np.minimum(a, 0)))

    def dec(x):
        a1 = W1 @ x + b1
        h1 = elu(a1)
        T1 = delu(a1)[:, None] * W1
        a2 = W2 @ h1 + b2
        h2 = elu(a2)
        T2 = delu(a2)[:, None] * (W2 @ T1)
        y = uref + scale * (W3 @ h2 + b3)
        D = scale[:, None] * (W3 @ T2)
        return y, D
    return dec


def lspg_bdf(problem, s2st, decoder, x0, dt, n_steps, order=1, iters=5, tol=1e-10):
    """problem: oracle Problem on the sample mesh; returns (x, [x per step])."""
    sd = sample_dofs(s2st, problem.ndpc)
    x = np.array(x0, dtype=np.float64)
    traj = []
    ynm1 = None
    for step in range(1, n_steps + 1):
        yn = decoder(x)[0][sd]
        two = order == 2 and step > 1
        cf, cn, cnm1 = ((-1. * (2. / 3.) * dt, -1. * (4. / 3.), 1. / 3.) if two else (-1. * dt, -1., 0.))
        for _ in range(iters):
            y, D = decoder(x)
            V, rp, ci, jv = problem.velocity_and_jacobian(y)
            J = sp.csr_matrix((jv, ci, rp), shape=(len(rp) - 1, len(y)))
            helper = 1. * y[sd] + cn * yn + cnm1 * ynm1 if two else 1. * y[sd] + cn * yn
            R = cf * V + helper
            JR = cf * (J @ D) + D[sd]
            dx = np.linalg.solve(JR.T @ JR, JR.T @ R)
            x = x - dx
            if np.linalg.norm(dx) < tol:
                break
        ynm1 = yn
        traj.append(x.copy())
    return x, traj


def lspg_bdf1(problem, s2st, decoder, x0, dt, n_steps, iters=5, tol=1e-10):
    return lspg_bdf(problem, s2st, decoder, x0, dt, n_steps, 1, iters, tol)
