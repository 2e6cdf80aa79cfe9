"""Shared test fixtures.

Markers: ``gpu`` -- needs a CUDA device (GB300); everything else runs on CPU.
"""
from __future__ import annotations

import importlib.util
import json
import os
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
PKG_DIR = os.path.join(REPO, "pressio-demoapps_gb300")
ORACLE_DIR = os.path.join(REPO, "oracle")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_package():
    """Import the pressio-demoapps_gb300 directory as module ``pda_gb300``."""
    if "pda_gb300" in sys.modules:
        return sys.modules["pda_gb300"]
    spec = importlib.util.spec_from_file_location("pda_gb300", os.path.join(PKG_DIR, "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pda_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def ensure_built():
    """Build libpda_gb300.so if it is missing (nvcc cross-compiles without a GPU)."""
    pkg = load_package()
    if not os.path.exists(pkg.LIB_PATH):
        spec = importlib.util.spec_from_file_location("pda_build_lib", os.path.join(PKG_DIR, "build_lib.py"))
        b = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(b)
        b.build()
    return pkg


@pytest.fixture(scope="session")
def pda():
    return ensure_built()


@pytest.fixture(scope="session")
def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def create_case_problem(pda, m, mesh, stream=None):
    """The library problem of a golden case; cross-shock parameters go through
    the cross-shock factory, the only way the reference accepts them."""
    scheme = pda.InviscidFluxReconstruction(m["scheme"])
    if m["family"] == 1 and m["problem"] == 7 and m.get("params"):
        q = m["params"]
        return pda.create_cross_shock_problem(mesh, scheme, q.get("crossShockDensity", 0.1),
                                              q.get("crossShockInletXVel", 10.0),
                                              q.get("crossShockBottomYVel", 1.0), stream=stream)
    enum = [pda.Euler1d, pda.Euler2d, pda.Euler3d, pda.Swe2d][m["family"]](m["problem"])
    return pda.create_problem(mesh, enum, scheme, m["icflag"], m.get("params") or None, stream=stream)


def golden_case(name):
    return dict(np.load(os.path.join(GOLDEN, "cases", name + ".npz")))


def mesh_dir(name):
    return os.path.join(GOLDEN, "meshes", name)


@pytest.fixture(scope="session")
def oracle():
    """The C restatement (oracle/liboracle.so), built on demand."""
    sys.path.insert(0, ORACLE_DIR)
    import oracle_py  # noqa: E402
    return oracle_py.load()


def v_close(got, ref, ndpc, rtol=1e-13, floor_frac=1e-3):
    """Per-cell velocity check |g - r| <= rtol * max(|r|, floor_frac * ||r_field||_inf):
    the floor is needed because the reference velocity is exactly zero in
    uniform regions."""
    g = np.asarray(got).reshape(-1, ndpc)
    r = np.asarray(ref).reshape(-1, ndpc)
    # NaN (a negative reconstructed pressure in the reference) must appear in
    # the same places; the finite values are compared
    if not np.array_equal(np.isnan(g), np.isnan(r)):
        return False, float("inf")
    g, r = np.nan_to_num(g, nan=0.0), np.nan_to_num(r, nan=0.0)
    fmax = np.max(np.abs(r), axis=0)
    tol = rtol * np.maximum(np.abs(r), floor_frac * fmax[None, :])
    bad = np.abs(g - r) > tol
    return (not bad.any()), float(np.max(np.abs(g - r) / np.maximum(tol / rtol, 1e-300)))


def j_close(got, ref, rowptr, rtol=1e-12, floor_frac=1e-3):
    """CSR value check with a per-row floor (same rule as v_close, rows of J)."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    if not np.array_equal(np.isnan(got), np.isnan(ref)):
        return False, float("inf")
    got, ref = np.nan_to_num(got, nan=0.0), np.nan_to_num(ref, nan=0.0)
    if len(ref) == 0:
        return True, 0.0
    rowptr = np.asarray(rowptr, dtype=np.int64)
    counts = np.diff(rowptr)
    absr = np.abs(ref)
    rmax = np.zeros(len(counts))
    nz = counts > 0
    rmax[nz] = np.maximum.reduceat(absr, rowptr[:-1][nz])
    tol = rtol * np.maximum(absr, floor_frac * np.repeat(rmax, counts))
    tol = np.maximum(tol, 1e-300)
    err = np.abs(got - ref)
    bad = err > tol
    return (not bad.any()), float(np.max(err / tol * rtol))
