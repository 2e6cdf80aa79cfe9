"""CPU tests of the C ABI library: every symbol declared in include/*.h is
exported, the native mesh generators reproduce the reference's mesh scripts
and the reference tests' mesh golds byte for byte, host-side problem logic
(parameters, initial conditions, CSR pattern) matches the reference, and
invalid input fails with a status code instead of crashing.  No kernel runs."""
from __future__ import annotations

import filecmp
import glob
import importlib.util
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, REPO, create_case_problem, golden_case, mesh_dir

MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_library_exports_every_declared_symbol(pda):
    L = pda.lib()
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(pda_[a-z0-9_]+)\s*\(", src))
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert L.pda_version().decode().startswith("pda_gb300")


def _parse_args(args):
    toks = args.split()
    n = [int(x) for x in toks[toks.index("-n") + 1:toks.index("--bounds")]]
    bi = toks.index("--bounds") + 1
    bounds = []
    while bi < len(toks) and re.fullmatch(r"[-+]?\d+(\.\d*)?", toks[bi]):
        bounds.append(float(toks[bi]))
        bi += 1
    st = int(toks[toks.index("-s") + 1])
    per = toks[toks.index("--periodic") + 1:] if "--periodic" in toks else []
    return n, bounds, st, ["x" in per, "y" in per, "z" in per]


@pytest.mark.parametrize("name", sorted(_make_golden().FULL_MESHES))
def test_native_generator_matches_reference_script(pda, tmp_path, name):
    n, bounds, st, per = _parse_args(_make_golden().FULL_MESHES[name])
    m = pda.create_full_mesh(n, bounds, st, per)
    m.write(str(tmp_path))
    for f in ("info.dat", "connectivity.dat", "coordinates.dat"):
        assert filecmp.cmp(os.path.join(tmp_path, f), os.path.join(mesh_dir(name), f), shallow=False), f


MESH_GOLD = json.load(open(os.path.join(GOLDEN, "gold", "mesh_generation", "args.json")))


@pytest.mark.parametrize("name", sorted(MESH_GOLD))
def test_native_generator_matches_reference_mesh_golds(pda, tmp_path, name):
    """tests_mesh/mesh_generation_full_{1,2,3}d of the reference: info.dat
    identical line by line, connectivity identical, coordinates within 1e-10
    (compare_mesh_files.py)."""
    a = MESH_GOLD[name]
    m = pda.create_full_mesh(a["n"][: a["dim"]] if a["dim"] > 1 else [a["n"][0], 1], a["bounds"], a["stencil"],
                             a["periodic"][: a["dim"]])
    m.write(str(tmp_path))
    gd = os.path.join(GOLDEN, "gold", "mesh_generation", name)
    assert open(os.path.join(tmp_path, "info.dat")).read() == open(os.path.join(gd, "info.dat")).read()
    assert np.array_equal(np.loadtxt(os.path.join(tmp_path, "connectivity.dat")),
                          np.loadtxt(os.path.join(gd, "connectivity.dat")))
    c1 = np.loadtxt(os.path.join(tmp_path, "coordinates.dat"))
    c2 = np.loadtxt(os.path.join(gd, "coordinates.dat"))
    assert np.allclose(c1[:, 0], c2[:, 0]) and np.allclose(c1[:, 1:], c2[:, 1:], atol=1e-10)


@pytest.mark.parametrize("name", sorted(_make_golden().SAMPLE_MESHES))
def test_native_sample_mesh_matches_reference_script(pda, tmp_path, name):
    full, _ = _make_golden().SAMPLE_MESHES[name]
    fm = pda.load_cellcentered_uniform_mesh(mesh_dir(full))
    gids = np.loadtxt(os.path.join(mesh_dir(name), "sample_mesh_gids.dat"), dtype=np.int64)
    sm, st = pda.create_sample_mesh(fm, gids)
    sm.write(str(tmp_path))
    for f in ("info.dat", "connectivity.dat", "coordinates.dat"):
        assert filecmp.cmp(os.path.join(tmp_path, f), os.path.join(mesh_dir(name), f), shallow=False), f
    assert np.array_equal(st, np.loadtxt(os.path.join(mesh_dir(name), "stencil_mesh_gids.dat"), dtype=np.int64))


def test_mesh_loader_and_classification(pda):
    """Inner / near-boundary row lists and full periodicity (mesh_ccu.hpp:161-342)."""
    m = pda.load_cellcentered_uniform_mesh(mesh_dir("m2d_s7_20"))
    assert m.dimensionality() == 2 and m.stencilSize() == 7
    assert m.sampleMeshSize() == 400 and m.stencilMeshSize() == 400
    assert m.numCellsInner() == 14 * 14 and m.numCellsNearBd() == 400 - 196
    assert m.isStructured() and not m.isFullyPeriodic()
    assert m.dx() == 0.05 and m.dxInv() == 1.0 / 0.05
    p = pda.load_cellcentered_uniform_mesh(mesh_dir("m2d_s7_16_per"))
    assert p.isFullyPeriodic() and p.numCellsNearBd() == 0
    s = pda.load_cellcentered_uniform_mesh(mesh_dir("s2d_s7_10"))
    assert not s.isStructured()
    g = m.graph()
    assert g.shape == (400, 13) and g[0, 1] == -1 and g[0, 3] == 1


def test_missing_mesh_files_are_an_error_not_an_exit(pda, tmp_path):
    with pytest.raises(pda.PdaError) as e:
        pda.load_cellcentered_uniform_mesh(str(tmp_path))
    assert e.value.code == -2 and "info.dat" in str(e.value)


@pytest.mark.parametrize("case", sorted(MANIFEST))
def test_host_initial_condition_and_pattern(pda, case):
    """Initial condition (host formulas, reference operation order) and the
    CSR pattern (Eigen setFromTriplets order) are bit-exact."""
    m = MANIFEST[case]
    g = golden_case(case)
    mesh = pda.load_cellcentered_uniform_mesh(mesh_dir(m["mesh"]))
    p = create_case_problem(pda, m, mesh, stream=0)
    assert p.numDofPerCell() == m["ndpc"]
    assert np.array_equal(p.initialConditionHost(), g["U0"])
    rp, ci = p.jacobianPatternHost()
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colidx"])


def test_parameters_and_errors(pda):
    mesh = pda.load_cellcentered_uniform_mesh(mesh_dir("m2d_s7_25"))
    p = pda.create_problem(mesh, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1,
                           {"gravity": 7.0, "coriolis": -1.5, "pulseMagnitude": 0.2}, stream=0)
    assert p.gravity() == 7.0 and p.coriolis() == -1.5 and p.queryParameter("pulseMagnitude") == 0.2
    assert p.queryParameter("pulseX") == 1.0
    q = pda.create_slip_wall_swe_2d_problem(mesh, pda.InviscidFluxReconstruction.Weno5, 8.0, -2.0, 0.1, stream=0)
    assert q.gravity() == 8.0 and q.queryParameter("pulseMagnitude") == 0.1
    with pytest.raises(pda.PdaError):  # unknown name (the reference throws)
        pda.create_problem(mesh, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1, {"nope": 1.0}, stream=0)
    with pytest.raises(pda.PdaError):  # ic2 name with ic1
        pda.create_problem(mesh, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1, {"pulseX2": 1.0}, stream=0)
    with pytest.raises(pda.PdaError):  # invalid icFlag
        pda.create_problem(mesh, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 3, stream=0)
    with pytest.raises(pda.PdaError):  # mesh dimensionality mismatch
        pda.create_problem(mesh, pda.Euler1d.Sod, pda.InviscidFluxReconstruction.Weno5, stream=0)
    m3 = pda.load_cellcentered_uniform_mesh(mesh_dir("m2d_s3_25"))
    with pytest.raises(pda.PdaError):  # stencil too small for WENO5
        pda.create_problem(m3, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, stream=0)
    e2 = pda.load_cellcentered_uniform_mesh(mesh_dir("m2d_s7_20"))
    r = pda.create_problem(e2, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2,
                           {"riemannTopRightPressure": 1.2, "gamma": 1.3}, stream=0)
    assert r.gamma() == 1.3 and r.queryParameter("riemannTopRightPressure") == 1.2
    with pytest.raises(pda.PdaError):  # riemann IC2 validity check (euler_2d_initial_condition.hpp:333)
        bad = pda.create_problem(e2, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2,
                                 {"riemannTopRightPressure": 0.01}, stream=0)
        bad.initialConditionHost()
    with pytest.raises(pda.PdaError):  # PeriodicSmooth needs a fully periodic mesh
        pda.create_problem(e2, pda.Euler2d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5, stream=0)


def _mesh_equal(a, b):
    assert (a.dimensionality(), a.stencilSize(), a.sampleMeshSize(), a.stencilMeshSize()) == \
        (b.dimensionality(), b.stencilSize(), b.sampleMeshSize(), b.stencilMeshSize())
    assert a.isStructured() == b.isStructured() and a.isFullyPeriodic() == b.isFullyPeriodic()
    assert a.dx() == b.dx() and a.dxInv() == b.dxInv()
    for u, v in zip(a._arrays(), b._arrays()):
        assert u.dtype == v.dtype and np.array_equal(u, v)


@pytest.mark.parametrize("n,bounds,st,per", [
    ((40,), (-0.5, 0.5), 7, (False,)),
    ((24, 18), (0.0, 1.0, 0.0, 2.0), 5, (False, True)),
    ((12, 10, 8), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True)),
    ((9, 11, 6), (0.0, 1.0, 0.0, 1.0, 0.0, 1.0), 3, (False, False, False)),
])
def test_binary_mesh_round_trip(pda, tmp_path, n, bounds, st, per):
    """The library's binary mesh file gives back the mesh written, bit for
    bit: graph, coordinates, spacing, row classification and the structured
    descriptor (1D, 2D and 3D; periodic and bounded axes)."""
    m = pda.create_full_mesh(n, bounds, st, per)
    f = tmp_path / "mesh.bin"
    m.write_binary(f)
    _mesh_equal(pda.load_mesh_binary(f), m)


@pytest.mark.parametrize("name", ["m2d_s7_20", "s2d_s7_10", "m2d_s7_16_per"])
def test_binary_mesh_equals_text_mesh(pda, tmp_path, name):
    """A mesh read from the reference's text files (full, sample and periodic)
    and saved in the binary format loads back identical."""
    m = pda.load_cellcentered_uniform_mesh(mesh_dir(name))
    f = tmp_path / "mesh.bin"
    m.write_binary(f)
    _mesh_equal(pda.load_mesh_binary(f), m)


def test_binary_mesh_sample_round_trip(pda, tmp_path):
    full = pda.create_full_mesh((30, 20), (0.0, 1.0, 0.0, 1.0), 7)
    sm, _ = pda.create_sample_mesh(full, np.arange(0, 600, 7, dtype=np.int64))
    f = tmp_path / "sample.bin"
    sm.write_binary(f)
    _mesh_equal(pda.load_mesh_binary(f), sm)


def test_binary_mesh_rejects_bad_files(pda, tmp_path):
    """Missing, truncated, corrupt and foreign files are PDA_ERR_IO, never a
    crash or a silently wrong mesh."""
    m = pda.create_full_mesh((16, 16), (0.0, 1.0, 0.0, 1.0), 5)
    good = tmp_path / "good.bin"
    m.write_binary(good)
    data = good.read_bytes()
    cases = {
        "missing": None,
        "truncated": data[:-9],
        "extended": data + b"\0" * 8,
        "flipped": data[:300] + bytes([data[300] ^ 0x10]) + data[301:],
        "magic": b"XDAMESH1" + data[8:],
        "text": b"dim 2\n",
    }
    for name, blob in cases.items():
        f = tmp_path / (name + ".bin")
        if blob is not None:
            f.write_bytes(blob)
        with pytest.raises(pda.PdaError) as e:
            pda.load_mesh_binary(f)
        assert e.value.code == -2, name


@pytest.mark.gpu
def test_problem_on_binary_mesh_equals_text_mesh(pda, tmp_path):
    """A problem built on the binary-loaded mesh evaluates the same velocity
    and Jacobian as on the text-loaded mesh, bit for bit."""
    import torch
    m = MANIFEST["riemann_w5"]
    g = golden_case("riemann_w5")
    text = pda.load_cellcentered_uniform_mesh(mesh_dir(m["mesh"]))
    f = tmp_path / "mesh.bin"
    text.write_binary(f)
    binm = pda.load_mesh_binary(f)
    out = []
    for mesh in (text, binm):
        p = create_case_problem(pda, m, mesh)
        U = torch.from_numpy(g["U1"]).cuda()
        V = p.createVelocity()
        J = p.createJacobian()
        p.rightHandSideAndJacobian(U, 0.0, V, J)
        torch.cuda.synchronize()
        out.append((V.cpu().numpy(), J.values.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
