"""The library's point-wise numerics (csrc/numerics.cuh: WENO3/5 with and
without gradients, Rusanov fluxes and flux Jacobians), compiled for the host
without FMA contraction, against the oracle's restatement of the reference on
random inputs.  Values must agree bit for bit; the few documented deviations
(sqrt for pow(h, 0.5), a correctly rounded cube for pow(x, 3)) are expected
to agree bit for bit too except in pathological near-midpoint cases, which
random sampling does not hit.  CPU only."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, REPO


@pytest.fixture(scope="module")
def host_numerics(tmp_path_factory):
    out = tmp_path_factory.mktemp("numerics") / "libpdn.so"
    src = os.path.join(REPO, "tests", "numerics_host.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I" + os.path.join(PKG_DIR, "csrc"), "-o", str(out), src], check=True)
    return C.CDLL(str(out))


def vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _stencils(rng, n, width):
    """Mixture of smooth, discontinuous and nearly constant stencils."""
    base = rng.uniform(0.1, 3.0, (n, 1))
    kind = rng.integers(0, 3, n)
    q = np.empty((n, width))
    smooth = base + rng.uniform(-1, 1, (n, 1)) * np.linspace(-1, 1, width)[None, :] ** rng.integers(1, 3, (n, 1))
    jump = base + (np.arange(width)[None, :] >= rng.integers(1, width, (n, 1))) * rng.uniform(-2, 2, (n, 1))
    flat = base + rng.uniform(-1e-7, 1e-7, (n, width))
    q[kind == 0] = smooth[kind == 0]
    q[kind == 1] = jump[kind == 1]
    q[kind == 2] = flat[kind == 2]
    return np.ascontiguousarray(q)


@pytest.mark.parametrize("scheme,width", [("weno5", 6), ("weno3", 4)])
def test_weno_bitwise(oracle, host_numerics, scheme, width):
    rng = np.random.default_rng(1)
    Q = _stencils(rng, 20000, width)
    f_o = getattr(oracle.L, f"orc_{scheme}_face")
    f_h = getattr(host_numerics, f"pdn_{scheme}_face")
    g_o = getattr(oracle.L, f"orc_{scheme}_face_grad")
    g_h = getattr(host_numerics, f"pdn_{scheme}_face_grad")
    for fn in (f_o, f_h):
        fn.argtypes = [C.c_void_p, C.c_void_p]
    for fn in (g_o, g_h):
        fn.argtypes = [C.c_void_p] * 4
    mism = 0
    for q in Q:
        a, b = np.empty(2), np.empty(2)
        f_o(vp(q), vp(a))
        f_h(vp(q), vp(b))
        assert np.array_equal(a, b)
        ga, gb = np.empty(2), np.empty(2)
        gna, gpa, gnb, gpb = (np.empty(width) for _ in range(4))
        g_o(vp(q), vp(ga), vp(gna), vp(gpa))
        g_h(vp(q), vp(gb), vp(gnb), vp(gpb))
        assert np.array_equal(ga, gb)
        if not (np.array_equal(gna, gnb) and np.array_equal(gpa, gpb)):
            mism += 1
            assert np.allclose(gna, gnb, rtol=1e-12, atol=1e-14) and np.allclose(gpa, gpb, rtol=1e-12, atol=1e-14)
    # gradients go through pow(x, 3); glibc's pow is not always correctly rounded
    assert mism < len(Q) // 100, f"{mism} gradient mismatches"


@pytest.mark.parametrize("family,axes,nd,param", [(0, 1, 3, 1.4), (1, 2, 4, 1.4), (2, 3, 5, 1.4), (3, 2, 3, 9.8)])
def test_flux_and_flux_jacobian_bitwise(oracle, host_numerics, family, axes, nd, param):
    rng = np.random.default_rng(2 + family)
    fo, fh = oracle.L.orc_point_flux, host_numerics.pdn_point_flux
    for fn in (fo, fh):
        fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    fs = host_numerics.pdn_point_flux_split
    fs.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    for _ in range(5000):
        qL, qR = rng.uniform(-1, 1, nd), rng.uniform(-1, 1, nd)
        qL[0], qR[0] = rng.uniform(0.2, 2.0), rng.uniform(0.2, 2.0)
        if family != 3:
            kin = lambda q: 0.5 * np.sum(q[1:nd - 1] ** 2) / q[0]
            qL[-1] = kin(qL) + rng.uniform(0.5, 3.0)
            qR[-1] = kin(qR) + rng.uniform(0.5, 3.0)
        for ax in range(axes):
            F1, F2 = np.empty(nd), np.empty(nd)
            J = [np.empty(nd * nd) for _ in range(4)]
            fo(family, ax, vp(qL), vp(qR), param, vp(F1), vp(J[0]), vp(J[1]))
            fh(family, ax, vp(qL), vp(qR), param, vp(F2), vp(J[2]), vp(J[3]))
            # the axis-specialised flux differs at most in the sign of an exact zero
            assert np.array_equal(F1, F2)
            # the flux in two halves (face states on separate threads) is the same flux
            F3 = np.empty(nd)
            fs(family, ax, vp(qL), vp(qR), param, vp(F3))
            assert np.array_equal(F3, F2)
            # shallow-water Jacobians use sqrt for glibc's pow(h, 0.5): 1-ulp differences
            for a, b in ((J[0], J[2]), (J[1], J[3])):
                assert np.allclose(a, b, rtol=1e-13, atol=1e-15 * np.abs(a).max())
                if family != 3:
                    assert np.array_equal(a, b)
