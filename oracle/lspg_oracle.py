"""Test infrastructure only (the oracle): numpy restatement of hyper-reduced
LSPG with BDF1 and Gauss-Newton, the algorithm of Pressio's
LspgUnsteadyResidualJacobianPolicyHypRed
(tests_cpp/pressio/include/pressio/rom/impl/lspg_unsteady_rj_policy_hypred.hpp:
180-264; BDF1 constants c_np1 = 1, c_n = -1, c_f = -1 from
ode/ode_constants.hpp:61-63), over the C oracle's sample-mesh velocity and
Jacobian.  Imported by tests/ only.

Per step n -> n+1 and iteration, with y(x) the trial state on the stencil mesh
and D = dy/dx:
    R  = cf V(y) + (y - y_n)|sample,        cf = -dt
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


def lspg_bdf1(problem, s2st, decoder, x0, dt, n_steps, iters=5, tol=1e-10):
    """problem: oracle Problem on the sample mesh; returns (x, [x per step])."""
    sd = sample_dofs(s2st, problem.ndpc)
    x = np.array(x0, dtype=np.float64)
    traj = []
    for _ in range(n_steps):
        yn = decoder(x)[0][sd]
        for _ in range(iters):
            y, D = decoder(x)
            V, rp, ci, jv = problem.velocity_and_jacobian(y)
            J = sp.csr_matrix((jv, ci, rp), shape=(len(rp) - 1, len(y)))
            R = -dt * V + (y[sd] - yn)
            JR = -dt * (J @ D) + D[sd]
            dx = np.linalg.solve(JR.T @ JR, JR.T @ R)
            x = x - dx
            if np.linalg.norm(dx) < tol:
                break
        traj.append(x.copy())
    return x, traj
