"""The C++ drop-in: a program written against include/pda_gb300.hpp (the
wrapper with the reference's PublicProblemEigenMixinCpp method names), built
with the system compilers and run as the reference's own explicit Riemann
test runs (tests_cpp/eigen_2d_euler_riemann_explicit/main.cc: Riemann IC2,
SSP-RK3, dt = 0.01, 60 steps).  Its final states, from a host-driven stepper
over the host-vector right-hand side and from the device stepper, are
checked against the reference test's rho/p golds.

CPU: the program compiles (syntax and types) against the headers.
GPU: it builds, links libpda_gb300.so and reproduces the golds."""
from __future__ import annotations

import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO, mesh_dir

SRC = os.path.join(REPO, "tests", "cpp", "riemann_ssprk3_consumer.cpp")
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "pressio-demoapps_gb300", "lib")
CUDA_INC = "/usr/local/cuda/include"
TRAJ = json.load(open(os.path.join(GOLDEN, "gold", "trajectories.json")))


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def test_consumer_compiles_against_the_headers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    cmd = [cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I" + INCLUDE, "-I" + CUDA_INC, SRC]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


def _pressure(D):
    rho = D[:, 0]
    u, v = D[:, 1] / rho, D[:, 2] / rho
    return rho, ((5. + 2.) / 5. - 1.) * (D[:, 3] - rho * (u ** 2 + v ** 2) * 0.5)


@pytest.mark.gpu
def test_consumer_reproduces_reference_riemann_golds(pda, tmp_path):
    exe = str(tmp_path / "consumer")
    cmd = [_nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, SRC, "-o", exe,
           "-L" + LIBDIR, "-lpda_gb300", "-Xlinker", "-rpath=" + LIBDIR]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    for name in ("riemann_firstorder", "riemann_weno3", "riemann_weno5"):
        t = TRAJ[name]
        oh, od = str(tmp_path / (name + "_host.bin")), str(tmp_path / (name + "_dev.bin"))
        r = subprocess.run([exe, mesh_dir(t["mesh"]), str(t["scheme"]), repr(t["dt"]), str(t["steps"]), oh, od],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        gold = np.load(os.path.join(GOLDEN, "gold", name + ".npz"))
        Dh = np.fromfile(oh, dtype=np.float64).reshape(-1, 4)
        Dd = np.fromfile(od, dtype=np.float64).reshape(-1, 4)
        # the host stepper rounds its updates like the device stepper
        assert np.array_equal(Dh, Dd), f"{name}: host and device steppers differ"
        for D in (Dh, Dd):
            rho, pr = _pressure(D)
            assert np.allclose(rho, gold["rho"], rtol=t["rtol"], atol=t["atol"]), name
            assert np.allclose(pr, gold["p"], rtol=t["rtol"], atol=t["atol"]), name
