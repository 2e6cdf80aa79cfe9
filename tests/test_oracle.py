"""The oracle (C restatement) pinned against the reference's own results:
golden cases generated by the reference itself, the reference tests' WENO
known answers and trajectory golds.  CPU only."""
from __future__ import annotations

import filecmp
import importlib.util
import json
import os
import re
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ORACLE_DIR, golden_case, mesh_dir

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


def _mesh_gen():
    sys.path.insert(0, ORACLE_DIR)
    import mesh_gen
    return mesh_gen


def generated_mesh(oracle, t):
    """The case's full mesh from the oracle's restatement of the reference's
    create_full_mesh.py (oracle/mesh_gen.py)."""
    return _mesh_gen().full_mesh(tuple(t["n"]), tuple(t["bounds"]), t["stencil"], orc=oracle).oracle_mesh(oracle)


def _full_mesh_args():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    out = {}
    for name, args in m.FULL_MESHES.items():
        toks = args.split()
        n = [int(x) for x in toks[toks.index("-n") + 1:toks.index("--bounds")]]
        bi = toks.index("--bounds") + 1
        bounds = []
        while bi < len(toks) and re.fullmatch(r"[-+]?\d+(\.\d*)?", toks[bi]):
            bounds.append(float(toks[bi]))
            bi += 1
        st = int(toks[toks.index("-s") + 1])
        per = toks[toks.index("--periodic") + 1:] if "--periodic" in toks else []
        if len(n) == 2 and n[1] == 1:
            n = n[:1]
        out[name] = (n, bounds, st, ["x" in per, "y" in per, "z" in per][:len(n)])
    return out


FULL_MESH_ARGS = _full_mesh_args()


@pytest.mark.parametrize("name", sorted(FULL_MESH_ARGS))
def test_oracle_mesh_generator_matches_reference_script(oracle, tmp_path, name):
    """oracle/mesh_gen.py writes the reference script's three files byte for
    byte (meshes made by meshing_scripts/create_full_mesh.py itself)."""
    n, bounds, st, per = FULL_MESH_ARGS[name]
    m = _mesh_gen().full_mesh(n, bounds, st, per)
    m.write(str(tmp_path))
    for f in ("info.dat", "connectivity.dat", "coordinates.dat"):
        assert filecmp.cmp(os.path.join(tmp_path, f), os.path.join(mesh_dir(name), f), shallow=False), f
    # and the arrays handed to the oracle are what the oracle's file reader gets
    om = oracle.mesh_load(mesh_dir(name))
    assert om.counts == m.oracle_mesh(oracle).counts


MESH_GOLD = json.load(open(os.path.join(GOLDEN, "gold", "mesh_generation", "args.json")))


@pytest.mark.parametrize("name", sorted(MESH_GOLD))
def test_oracle_mesh_generator_matches_reference_mesh_golds(tmp_path, name):
    """The reference's tests_mesh/mesh_generation_full_{1,2,3}d golds:
    info.dat identical, connectivity identical, coordinates within 1e-10."""
    a = MESH_GOLD[name]
    n = a["n"][: a["dim"]]
    m = _mesh_gen().full_mesh(n, a["bounds"][: 2 * a["dim"]], a["stencil"], a["periodic"][: a["dim"]])
    m.write(str(tmp_path))
    gd = os.path.join(GOLDEN, "gold", "mesh_generation", name)
    assert open(os.path.join(tmp_path, "info.dat")).read() == open(os.path.join(gd, "info.dat")).read()
    assert np.array_equal(np.loadtxt(os.path.join(tmp_path, "connectivity.dat")),
                          np.loadtxt(os.path.join(gd, "connectivity.dat")))
    c1 = np.loadtxt(os.path.join(tmp_path, "coordinates.dat"))
    c2 = np.loadtxt(os.path.join(gd, "coordinates.dat"))
    assert np.allclose(c1[:, 0], c2[:, 0]) and np.allclose(c1[:, 1:], c2[:, 1:], atol=1e-10)


def test_oracle_mesh_generator_round_trip_in_c(oracle):
    """The oracle's C round trip of "%.14f" equals Python's on a large mesh."""
    mg = _mesh_gen()
    a = mg.full_mesh((64, 48), (-5.0, 5.0, 0.0, 1.0), 7, orc=oracle)
    b = mg.full_mesh((64, 48), (-5.0, 5.0, 0.0, 1.0), 7)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


@pytest.mark.parametrize("name", sorted(GENTRAJ))
def test_oracle_generated_mesh_gold(oracle, name):
    """Golds of the reference tests whose meshes are regenerated here: the
    Python tests (their driver's SSP-RK3 update order, ``ssprk3_py``) and the
    3D Sedov symmetry runs (Pressio's order, whole state)."""
    t = GENTRAJ[name]
    p = oracle.problem(generated_mesh(oracle, t), t["family"], t["problem"], t["scheme"], t["icflag"])
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
