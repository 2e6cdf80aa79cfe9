"""Generate the hyper-reduced LSPG golden trajectories (tests/golden/lspg/)
from the reference itself: oracle/_ref/lspg_ref drives the vendored Pressio's
hyper-reduced LSPG (BDF1 and BDF2, Gauss-Newton with a fixed number of
iterations) over the reference's own shallow-water slip-wall problem on a
sample mesh made by the reference's create_sample_mesh.py
(tests/golden/meshes/s2d_s7_20: the cells of the reference test
eigen_2d_swe_jacobian_fd_with_sample_mesh on the 20x20 stencil-7 mesh).

Usage:  PDA_REFERENCE=<checkout> python tests/golden/make_lspg_golden.py
(builds oracle/_ref/lspg_ref with `make -C oracle lspgref REF=...`)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PDA_REFERENCE", "")
OUT = os.path.join(HERE, "lspg")
MESH = os.path.join(HERE, "meshes", "s2d_s7_20")
EXE = os.path.join(REPO, "oracle", "_ref", "lspg_ref")

# name -> (order, gn iterations, dt, steps, k, seed, (gravity, coriolis, pulse))
CASES = {
    "swe_s2d_s7_20_bdf1": (1, 6, 0.01, 6, 6, 3, (7.0, -2.0, 0.15)),
    "swe_s2d_s7_20_bdf2": (2, 6, 0.01, 6, 6, 3, (7.0, -2.0, 0.15)),
    "swe_s2d_s7_20_bdf2_k4_dt02": (2, 4, 0.02, 5, 4, 11, (9.0, -3.5, 0.18)),
}


def sample_to_stencil():
    sm = np.loadtxt(os.path.join(MESH, "sample_mesh_gids.dat"), dtype=np.int64)
    st = np.loadtxt(os.path.join(MESH, "stencil_mesh_gids.dat"), dtype=np.int64)
    return np.searchsorted(st, sm).astype(np.int64), len(st)


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "include", "pressiodemoapps")):
        sys.exit("set PDA_REFERENCE to a pressio-demoapps checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "lspgref", f"REF={REF}"], check=True)
    os.makedirs(OUT, exist_ok=True)
    s2st, nst_cells = sample_to_stencil()
    nst = 3 * nst_cells
    for name, (order, iters, dt, steps, k, seed, (g, f, a)) in CASES.items():
        rng = np.random.default_rng(seed)
        phi, _ = np.linalg.qr(rng.normal(0, 1, (nst, k)))
        phi = np.ascontiguousarray(phi * 0.3)
        uref = np.zeros(nst)
        uref[0::3] = 1.0
        x0 = rng.uniform(-0.1, 0.1, k)
        with tempfile.TemporaryDirectory() as d:
            paths = {n: os.path.join(d, n) for n in ("s2st", "phi", "uref", "x0", "out")}
            s2st.tofile(paths["s2st"])
            phi.tofile(paths["phi"])
            uref.tofile(paths["uref"])
            x0.tofile(paths["x0"])
            subprocess.run([EXE, MESH, paths["s2st"], paths["phi"], paths["uref"], paths["x0"], str(k), repr(dt),
                            str(steps), str(order), str(iters), repr(g), repr(f), repr(a), paths["out"]], check=True)
            traj = np.fromfile(paths["out"], dtype=np.float64).reshape(-1, k)
        # the observer also sees the initial state
        if traj.shape[0] == steps + 1:
            traj = traj[1:]
        assert traj.shape == (steps, k), traj.shape
        # Pressio's Stop::AfterMaxIters evaluates the operators maxIters times
        # and stops before applying the last correction: iters - 1 updates
        np.savez(os.path.join(OUT, name + ".npz"), s2st=s2st, phi=phi, uref=uref, x0=x0, traj=traj,
                 order=order, iters=iters, updates=iters - 1, dt=dt, steps=steps, params=np.array([g, f, a]))
        print(name, traj[-1])


if __name__ == "__main__":
    main()
