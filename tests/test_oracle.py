"""The oracle (C restatement) pinned against the reference's own results:
golden cases generated by the reference itself, the reference tests' WENO
known answers and trajectory golds.  CPU only."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_case, mesh_dir

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
TRAJ = json.load(open(os.path.join(GOLDEN, "gold", "trajectories.json")))


def test_weno_known_answers(oracle):
    kat = json.load(open(os.path.join(GOLDEN, "gold", "weno_kat.json")))
    assert np.all(np.abs(oracle.weno5(kat["weno5_q"]) - kat["weno5_gold"]) <= kat["tol"])
    assert np.all(np.abs(oracle.weno3(kat["weno3_q"]) - kat["weno3_gold"]) <= kat["tol"])


def _problem(oracle, m):
    om = oracle.mesh_load(mesh_dir(m["mesh"]))
    return oracle.problem(om, m["family"], m["problem"], m["scheme"], m["icflag"], m.get("params"))


@pytest.mark.parametrize("case", sorted(MANIFEST))
def test_oracle_bitwise_against_reference(oracle, case):
    """The restatement follows the reference's operation order; compiled
    without FMA contraction it reproduces the reference bit for bit."""
    m = MANIFEST[case]
    g = golden_case(case)
    p = _problem(oracle, m)
    assert (p.dofs_sample, p.dofs_stencil, p.nnz) == (m["dofs_sample"], m["dofs_stencil"], m["nnz"])
    t = m.get("t", 0.0)
    assert np.array_equal(p.initial_condition(), g["U0"])
    # NaN where the reference's reconstruction gives a negative pressure
    assert np.array_equal(p.velocity(g["U0"], t), g["V0"], equal_nan=True)
    assert np.array_equal(p.velocity(g["U1"], t), g["V1"], equal_nan=True)
    V, rp, ci, jv = p.velocity_and_jacobian(g["U1"], t)
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colidx"])
    assert np.array_equal(V, g["Vj"], equal_nan=True)
    assert np.array_equal(jv, g["jvals"], equal_nan=True)


@pytest.mark.parametrize("name", sorted(TRAJ))
def test_oracle_trajectory_gold(oracle, name):
    t = TRAJ[name]
    p = _problem(oracle, t)
    U = p.initial_condition()
    if name.startswith("riemann") and t["scheme"] == 2:
        pytest.skip("covered by the first-order and WENO3 Riemann cases (runtime)")
    (p.rk4 if t["stepper"] == "rk4" else p.ssprk3)(U, 0.0, t["dt"], t["steps"])
    if name.startswith("sod"):
        gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
        assert np.allclose(U, gold, rtol=t["rtol"], atol=t["atol"])
    elif name.startswith("riemann"):
        gold = np.load(os.path.join(GOLDEN, "gold", name + ".npz"))
        D = U.reshape(-1, 4)
        rho = D[:, 0]
        u, v = D[:, 1] / rho, D[:, 2] / rho
        pr = ((5. + 2.) / 5. - 1.) * (D[:, 3] - rho * (u ** 2 + v ** 2) * 0.5)
        assert np.allclose(rho, gold["rho"], rtol=t["rtol"], atol=t["atol"])
        assert np.allclose(pr, gold["p"], rtol=t["rtol"], atol=t["atol"])
    elif name.startswith(("cross", "dmr")):
        gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
        assert np.allclose(U.reshape(-1, 4)[:, 0], gold, rtol=t["rtol"], atol=t["atol"])
    else:
        gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
        assert np.allclose(U.reshape(-1, 3)[:, 0], gold, rtol=t["rtol"], atol=t["atol"])


GENTRAJ = json.load(open(os.path.join(GOLDEN, "gold", "trajectories_generated_mesh.json")))


def generated_mesh(pda, oracle, t):
    """The case's full mesh from the library's host-side generator (the
    reference's create_full_mesh.py layout), handed to the oracle."""
    mesh = pda.create_full_mesh(tuple(t["n"]), tuple(t["bounds"]), t["stencil"])
    g, x, y, z, _, _ = mesh._arrays()
    dim = len(t["n"])
    return oracle.mesh_from_arrays(dim, t["stencil"], g, x, y, z, (mesh.dx(), mesh.dy(), mesh.dz()))


@pytest.mark.parametrize("name", sorted(GENTRAJ))
def test_oracle_generated_mesh_gold(pda, oracle, name):
    """Golds of the reference tests whose meshes are regenerated here: the
    Python tests (their driver's SSP-RK3 update order, ``ssprk3_py``) and the
    3D Sedov symmetry runs (Pressio's order, whole state)."""
    t = GENTRAJ[name]
    p = oracle.problem(generated_mesh(pda, oracle, t), t["family"], t["problem"], t["scheme"], t["icflag"])
    U = p.initial_condition()
    (p.ssprk3_py if t["stepper"] == "ssprk3_py" else p.ssprk3)(U, 0.0, t["dt"], t["steps"])
    gold = np.load(os.path.join(GOLDEN, "gold", name + ".npy"))
    got = U.reshape(-1, p.ndpc)[:, 0] if t["field"] == "rho" else U
    assert np.allclose(got, gold, rtol=t["rtol"], atol=t["atol"])


@pytest.mark.parametrize("case", sorted(MANIFEST))
def test_correctly_rounded_cube_stays_within_the_jacobian_tolerance(oracle, case):
    """The library evaluates the reference's pow(x, 3.) as a correctly rounded
    cube.  Evaluated that way, the oracle's Jacobian stays within 1e-12 of the
    row scale of the reference's (the case's own tolerance across the double
    Mach reflection's shock; velocities are unaffected)."""
    from conftest import j_close
    m = MANIFEST[case]
    g = golden_case(case)
    oracle.set_cube_mode(1)
    try:
        p = _problem(oracle, m)
        V, rp, ci, jv = p.velocity_and_jacobian(g["U1"], m.get("t", 0.0))
    finally:
        oracle.set_cube_mode(0)
    assert np.array_equal(V, g["Vj"], equal_nan=True)
    ok, worst = j_close(jv, g["jvals"], rp, rtol=m.get("jtol", 1e-12), floor_frac=1.0)
    assert ok, worst
