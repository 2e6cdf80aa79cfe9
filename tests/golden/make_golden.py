"""Generate the golden fixtures under tests/golden/ from the reference.

Runs only where a reference checkout exists; its location comes from the
environment variable PDA_REFERENCE (required).  It
  1. runs the reference's own mesh scripts (meshing_scripts/create_full_mesh.py,
     create_sample_mesh.py) into tests/golden/meshes/<name>/,
  2. evaluates the reference itself through oracle/_ref/libpdaref.so (built by
     ``make -C oracle ref`` from the reference headers) on seeded inputs and
     stores initial conditions, velocities and CSR Jacobians in
     tests/golden/cases/<case>.npz,
  3. copies the reference tests' own known answers (WENO KATs, Sod / Riemann /
     shallow-water trajectory golds, mesh-generator golds) into
     tests/golden/gold/, checking on the way that the reference shim
     reproduces them.

Usage:  PDA_REFERENCE=<checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PDA_REFERENCE", "")
MESHES = os.path.join(HERE, "meshes")
CASES = os.path.join(HERE, "cases")
GOLD = os.path.join(HERE, "gold")
SEED = 20261203

# name -> create_full_mesh.py arguments
FULL_MESHES = {
    "m1d_s3_100": "-n 100 1 --bounds -0.5 0.5 -s 3",
    "m1d_s5_100": "-n 100 1 --bounds -0.5 0.5 -s 5",
    "m1d_s7_100": "-n 100 1 --bounds -0.5 0.5 -s 7",
    "m1d_s7_7": "-n 7 1 --bounds -0.5 0.5 -s 7",
    "m1d_s7_40_per": "-n 40 1 --bounds -1.0 1.0 -s 7 --periodic x",
    "m2d_s3_20": "-n 20 20 --bounds 0.0 1.0 0.0 1.0 -s 3",
    "m2d_s5_20": "-n 20 20 --bounds 0.0 1.0 0.0 1.0 -s 5",
    "m2d_s7_20": "-n 20 20 --bounds 0.0 1.0 0.0 1.0 -s 7",
    "m2d_s7_13x11_perx": "-n 13 11 --bounds 0.0 1.0 0.0 1.0 -s 7 --periodic x",
    "m2d_s7_16_per": "-n 16 16 --bounds -1.0 1.0 -1.0 1.0 -s 7 --periodic x y",
    "m2d_s7_6_per": "-n 6 6 --bounds -1.0 1.0 -1.0 1.0 -s 7 --periodic x y",
    "m2d_s3_25": "-n 25 25 --bounds -5.0 5.0 -5.0 5.0 -s 3",
    "m2d_s5_25": "-n 25 25 --bounds -5.0 5.0 -5.0 5.0 -s 5",
    "m2d_s7_25": "-n 25 25 --bounds -5.0 5.0 -5.0 5.0 -s 7",
    "m2d_s3_10": "-n 10 10 --bounds 0.0 1.0 0.0 1.0 -s 3",
    "m2d_s5_10": "-n 10 10 --bounds 0.0 1.0 0.0 1.0 -s 5",
    "m2d_s7_10": "-n 10 10 --bounds 0.0 1.0 0.0 1.0 -s 7",
    "m2d_s7_20_per_kh": "-n 20 20 --bounds -5.0 5.0 -5.0 5.0 -s 7 --periodic x y",
    "m2d_s7_21_sedov": "-n 21 21 --bounds -1.2 1.2 -1.2 1.2 -s 7",
    "m2d_s7_16_sedsym": "-n 16 16 --bounds 0.0 1.2 0.0 1.2 -s 7",
    "m2d_s5_16_sedsym": "-n 16 16 --bounds 0.0 1.2 0.0 1.2 -s 5",
    "m2d_s3_16_sedsym": "-n 16 16 --bounds 0.0 1.2 0.0 1.2 -s 3",
    "m2d_s7_24x12_nshock": "-n 24 12 --bounds 0.0 2.0 0.0 1.0 -s 7",
    "m2d_s5_24x12_nshock": "-n 24 12 --bounds 0.0 2.0 0.0 1.0 -s 5",
    # cross-shock and double-Mach-reflection meshes of the reference's explicit tests
    # (tests_cpp/eigen_2d_euler_{cross_shock,double_mach_reflection}_explicit/test.cmake)
    "m2d_s3_40x20_cross": "-n 40 20 --bounds 0.0 2.0 0.0 1.0 -s 3",
    "m2d_s5_40x20_cross": "-n 40 20 --bounds 0.0 2.0 0.0 1.0 -s 5",
    "m2d_s7_40x20_cross": "-n 40 20 --bounds 0.0 2.0 0.0 1.0 -s 7",
    "m2d_s3_60x15_dmr": "-n 60 15 --bounds 0.0 4.0 0.0 1.0 -s 3",
    "m2d_s5_60x15_dmr": "-n 60 15 --bounds 0.0 4.0 0.0 1.0 -s 5",
    "m2d_s7_60x15_dmr": "-n 60 15 --bounds 0.0 4.0 0.0 1.0 -s 7",
    # 3D Sedov symmetry (tests_cpp/eigen_3d_euler_sedov_symmetry/test.cmake bounds)
    "m3d_s3_8_sedov": "-n 8 8 8 --bounds 0.0 0.4 0.0 0.4 0.0 0.4 -s 3",
    "m3d_s5_8_sedov": "-n 8 8 8 --bounds 0.0 0.4 0.0 0.4 0.0 0.4 -s 5",
    "m3d_s5_6x5x7_sedov": "-n 6 5 7 --bounds 0.0 0.4 0.0 0.4 0.0 0.4 -s 5",
    "m3d_s3_8_per": "-n 8 8 8 --bounds -1.0 1.0 -1.0 1.0 -1.0 1.0 -s 3 --periodic x y z",
    "m3d_s5_8_per": "-n 8 8 8 --bounds -1.0 1.0 -1.0 1.0 -1.0 1.0 -s 5 --periodic x y z",
    "m3d_s5_6x5x7_per": "-n 6 5 7 --bounds -1.0 1.0 -1.0 1.0 -1.0 1.0 -s 5 --periodic x y z",
}

# sample meshes: name -> (full mesh, gids source)
SAMPLE_MESHES = {
    "s2d_s3_10": ("m2d_s3_10", "tests_cpp/eigen_2d_euler_sample_mesh_test1/firstorder/sample_mesh_gids.dat"),
    "s2d_s5_10": ("m2d_s5_10", "tests_cpp/eigen_2d_euler_sample_mesh_test1/weno3/sample_mesh_gids.dat"),
    "s2d_s7_10": ("m2d_s7_10", "tests_cpp/eigen_2d_euler_sample_mesh_test1/weno5/sample_mesh_gids.dat"),
    "s2d_s7_20": ("m2d_s7_20", "tests_cpp/eigen_2d_swe_jacobian_fd_with_sample_mesh/sample_mesh_gids.dat"),
    "s2d_s7_25_rand": ("m2d_s7_25", "random:40"),
    "s2d_s7_16_sedsym_rand": ("m2d_s7_16_sedsym", "random:40"),
    "s2d_s7_60x15_dmr_rand": ("m2d_s7_60x15_dmr", "random:60"),
    "s2d_s5_40x20_cross_rand": ("m2d_s5_40x20_cross", "random:50"),
    "s3d_s5_8_sedov_rand": ("m3d_s5_8_sedov", "random:40"),
}

# case -> (mesh, family, problem, scheme, icflag, params)
E1, E2, E3, SW = 0, 1, 2, 3
CASE_LIST = {
    "sod_fo": ("m1d_s3_100", E1, 1, 0, 1, {}),
    "sod_w3": ("m1d_s5_100", E1, 1, 1, 1, {}),
    "sod_w5": ("m1d_s7_100", E1, 1, 2, 1, {}),
    "sod_w5_s7_fo": ("m1d_s7_100", E1, 1, 0, 1, {}),
    "sod_w5_tiny": ("m1d_s7_7", E1, 1, 2, 1, {}),
    "lax_w5": ("m1d_s7_100", E1, 2, 2, 1, {}),
    "e1d_smooth_w5": ("m1d_s7_40_per", E1, 0, 2, 1, {}),
    "riemann_fo": ("m2d_s3_20", E2, 4, 0, 2, {}),
    "riemann_w3": ("m2d_s7_20", E2, 4, 1, 2, {}),
    "riemann_w5": ("m2d_s7_20", E2, 4, 2, 2, {}),
    "riemann_w3_s5": ("m2d_s5_20", E2, 4, 1, 2, {}),
    "riemann_ic1_w5": ("m2d_s7_20", E2, 4, 2, 1, {}),
    "riemann_params_w5": ("m2d_s7_20", E2, 4, 2, 2,
                          {"riemannTopRightPressure": 1.2, "riemannTopRightDensity": 1.1,
                           "riemannBotLeftPressure": 0.05, "gamma": 1.3}),
    "riemann_perx_w5": ("m2d_s7_13x11_perx", E2, 4, 2, 2, {}),
    "e2d_smooth_w5": ("m2d_s7_16_per", E2, 0, 2, 1, {}),
    "e2d_smooth_w3": ("m2d_s7_16_per", E2, 0, 1, 1, {}),
    "e2d_smooth_w5_tiny": ("m2d_s7_6_per", E2, 0, 2, 1, {}),
    "swe_fo": ("m2d_s3_25", SW, 0, 0, 1, {}),
    "swe_w3": ("m2d_s5_25", SW, 0, 1, 1, {}),
    "swe_w5": ("m2d_s7_25", SW, 0, 2, 1, {}),
    "swe_ic2_w5": ("m2d_s7_25", SW, 0, 2, 2,
                   {"gravity": 7.5, "coriolis": -2.0, "pulseMagnitude1": 0.15, "pulseX2": 1.5}),
    "e3d_smooth_fo": ("m3d_s3_8_per", E3, 0, 0, 1, {}),
    "e3d_smooth_w3": ("m3d_s5_8_per", E3, 0, 1, 1, {}),
    "e3d_smooth_w3_odd": ("m3d_s5_6x5x7_per", E3, 0, 1, 1, {}),
    "sample_riemann_fo": ("s2d_s3_10", E2, 4, 0, 2, {}),
    "sample_riemann_w3": ("s2d_s5_10", E2, 4, 1, 2, {}),
    "sample_riemann_w5": ("s2d_s7_10", E2, 4, 2, 2, {}),
    "sample_swe_w5": ("s2d_s7_20", SW, 0, 2, 1, {}),
    "sample_swe_w5_rand": ("s2d_s7_25_rand", SW, 0, 2, 1, {"coriolis": -1.5}),
    "kh_w5": ("m2d_s7_20_per_kh", E2, 1, 2, 1, {}),
    "kh_w3": ("m2d_s7_20_per_kh", E2, 1, 1, 1, {}),
    "sedovfull_w5": ("m2d_s7_21_sedov", E2, 2, 2, 1, {}),
    "sedovsym_w5": ("m2d_s7_16_sedsym", E2, 3, 2, 1, {}),
    "sedovsym_w3": ("m2d_s5_16_sedsym", E2, 3, 1, 1, {}),
    "sedovsym_fo": ("m2d_s3_16_sedsym", E2, 3, 0, 1, {}),
    "sample_sedovsym_w5": ("s2d_s7_16_sedsym_rand", E2, 3, 2, 1, {}),
    "normalshock_w5": ("m2d_s7_24x12_nshock", E2, 5, 2, 1, {}),
    "normalshock_w3_mach": ("m2d_s5_24x12_nshock", E2, 5, 1, 1, {"mach": 4.0}),
    "dmr_fo": ("m2d_s3_60x15_dmr", E2, 6, 0, 1, {}),
    "dmr_w3": ("m2d_s5_60x15_dmr", E2, 6, 1, 1, {}),
    "dmr_w5": ("m2d_s7_60x15_dmr", E2, 6, 2, 1, {}),
    "dmr_w5_t0": ("m2d_s7_60x15_dmr", E2, 6, 2, 1, {}),
    "sample_dmr_w5": ("s2d_s7_60x15_dmr_rand", E2, 6, 2, 1, {}),
    "cross_fo": ("m2d_s3_40x20_cross", E2, 7, 0, 1, {}),
    "cross_w3": ("m2d_s5_40x20_cross", E2, 7, 1, 1, {}),
    "cross_w5": ("m2d_s7_40x20_cross", E2, 7, 2, 1, {}),
    "cross_params_w5": ("m2d_s7_40x20_cross", E2, 7, 2, 1,
                        {"crossShockDensity": 0.2, "crossShockInletXVel": 5.0, "crossShockBottomYVel": 2.0}),
    "sample_cross_w3": ("s2d_s5_40x20_cross_rand", E2, 7, 1, 1, {}),
    "sedov3d_fo": ("m3d_s3_8_sedov", E3, 1, 0, 1, {}),
    "sedov3d_w3": ("m3d_s5_8_sedov", E3, 1, 1, 1, {}),
    "sedov3d_w3_odd": ("m3d_s5_6x5x7_sedov", E3, 1, 1, 1, {}),
    "sample_sedov3d_w3": ("s3d_s5_8_sedov_rand", E3, 1, 1, 1, {}),
}

# evaluation time of a case (time-dependent ghost states: the double Mach
# reflection's top boundary follows the moving shock)
CASE_TIME = {"dmr_fo": 0.05, "dmr_w3": 0.08, "dmr_w5": 0.1, "sample_dmr_w5": 0.07}

# Jacobian tolerance (relative to the row's largest entry) where 1e-12 is
# below the problem's conditioning: across the Mach 10 shock of the double
# Mach reflection the WENO5 weight derivatives amplify a last-bit difference
# of x^3 (glibc pow versus a correctly rounded cube) to ~1e-11 of the row
# scale; the reference evaluated both ways differs by that much
CASE_JTOL = {"dmr_w5": 3e-11, "dmr_w5_t0": 3e-11}


def run(cmd):
    subprocess.run(cmd, shell=True, check=True, stdout=subprocess.DEVNULL)


def make_meshes():
    os.makedirs(MESHES, exist_ok=True)
    py = sys.executable
    for name, args in FULL_MESHES.items():
        d = os.path.join(MESHES, name)
        os.makedirs(d, exist_ok=True)
        run(f"{py} {REF}/meshing_scripts/create_full_mesh.py {args} --outDir {d}")
    rng = np.random.default_rng(SEED)
    for name, (full, src) in SAMPLE_MESHES.items():
        d = os.path.join(MESHES, name)
        os.makedirs(d, exist_ok=True)
        gfile = os.path.join(d, "sample_mesh_gids.dat")
        if src.startswith("random:"):
            k = int(src.split(":")[1])
            ncell = int(re.search(r"sampleMeshSize\s+(\d+)", open(os.path.join(MESHES, full, "info.dat")).read()).group(1))
            gids = np.sort(rng.choice(ncell, size=k, replace=False))
            np.savetxt(gfile, gids, fmt="%8d")
        else:
            shutil.copy(os.path.join(REF, src), gfile)
        run(f"{py} {REF}/meshing_scripts/create_sample_mesh.py --fullMeshDir {os.path.join(MESHES, full)} "
            f"--sampleMeshIndices {gfile} --outDir {d}")


class Ref:
    def __init__(self):
        path = os.path.join(REPO, "oracle", "_ref", "libpdaref.so")
        if not os.path.exists(path):
            subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={REF}"], check=True)
        L = C.CDLL(path)
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.POINTER(C.c_char_p), C.POINTER(C.c_double)]
        L.ref_last_error.restype = C.c_char_p
        for f in ("ref_destroy",):
            getattr(L, f).argtypes = [C.c_void_p]
        L.ref_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
        L.ref_ic.argtypes = [C.c_void_p, C.c_void_p]
        L.ref_velocity.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
        L.ref_velocity_and_jacobian.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_ssprk3.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_long]
        L.ref_rk4.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_long]
        L.ref_weno5.argtypes = [C.c_void_p, C.c_void_p]
        L.ref_weno3.argtypes = [C.c_void_p, C.c_void_p]
        self.L = L

    def create(self, mesh, fam, prob, scheme, ic, params):
        names = list(params)
        cn = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
        cv = (C.c_double * max(1, len(names)))(*[float(params[n]) for n in names])
        h = self.L.ref_create(os.path.join(MESHES, mesh).encode(), fam, prob, scheme, ic, len(names), cn, cv)
        if not h:
            raise RuntimeError(self.L.ref_last_error().decode())
        s = (C.c_long * 4)()
        self.L.ref_sizes(h, s)
        return h, tuple(s)


def vp(a):
    return a.ctypes.data_as(C.c_void_p)


def make_cases(ref: Ref):
    os.makedirs(CASES, exist_ok=True)
    rng = np.random.default_rng(SEED)
    manifest = {}
    for case, (mesh, fam, prob, scheme, ic, params) in CASE_LIST.items():
        h, (ndpc, ds, dst, nnz) = ref.create(mesh, fam, prob, scheme, ic, params)
        U0 = np.empty(dst)
        ref.L.ref_ic(h, vp(U0))
        noise = rng.uniform(-1e-3, 1e-3, dst)
        # Sedov states have an energy of ~6e-5 outside the blast: relative
        # noise keeps the pressure positive
        U1 = U0 * (1.0 + noise) if "sedov" in case else U0 + noise
        t = CASE_TIME.get(case, 0.0)
        V0 = np.empty(ds)
        V1 = np.empty(ds)
        ref.L.ref_velocity(h, vp(U0), t, vp(V0))
        ref.L.ref_velocity(h, vp(U1), t, vp(V1))
        Vj = np.empty(ds)
        rp = np.empty(ds + 1, dtype=np.int32)
        ci = np.empty(nnz, dtype=np.int32)
        jv = np.empty(nnz)
        ref.L.ref_velocity_and_jacobian(h, vp(U1), t, vp(Vj), vp(rp), vp(ci), vp(jv))
        ref.L.ref_destroy(h)
        np.savez_compressed(os.path.join(CASES, case + ".npz"), U0=U0, U1=U1, V0=V0, V1=V1, Vj=Vj,
                            rowptr=rp, colidx=ci, jvals=jv)
        manifest[case] = dict(mesh=mesh, family=fam, problem=prob, scheme=scheme, icflag=ic,
                              params=params, ndpc=ndpc, dofs_sample=ds, dofs_stencil=dst, nnz=nnz, t=t,
                              jtol=CASE_JTOL.get(case, 1e-12))
        print(f"case {case}: dofs {ds}/{dst} nnz {nnz}")
    return manifest


def extract_kat():
    """WENO known answers from tests_cpp/weno5/main.cc:12-25 and weno3/main.cc."""
    def nums(block):
        return [float(x) for x in re.findall(r"[-+]?\d+\.\d*(?:e[-+]?\d+)?", block)]
    src5 = open(os.path.join(REF, "tests_cpp/weno5/main.cc")).read()
    q5 = nums(re.search(r"vec_t q\{([^}]*)\}", src5).group(1))
    g5 = nums(re.search(r"goldF =\s*\{([^}]*)\}", src5).group(1))
    src3 = open(os.path.join(REF, "tests_cpp/weno3/main.cc")).read()
    q3 = nums(re.search(r"vec_t q\{([^}]*)\}", src3).group(1))
    g3 = nums(re.search(r"goldF =\s*\{([^}]*)\}", src3).group(1))
    return dict(weno5_q=q5, weno5_gold=g5, weno3_q=q3, weno3_gold=g3, tol=1e-13)


def make_gold(ref: Ref):
    os.makedirs(GOLD, exist_ok=True)
    kat = extract_kat()
    for tag, q, g in (("weno5", kat["weno5_q"], kat["weno5_gold"]), ("weno3", kat["weno3_q"], kat["weno3_gold"])):
        out = np.empty(4)
        getattr(ref.L, "ref_" + tag)(vp(np.array(q)), vp(out))
        assert np.all(np.abs(out - np.array(g)) <= 1e-13), (tag, out, g)
    json.dump(kat, open(os.path.join(GOLD, "weno_kat.json"), "w"), indent=1)

    traj = {}
    # Sod: RK4 dt=1e-3, 100 steps, last snapshot (tests_cpp/eigen_1d_euler_sod_explicit/main.cc)
    for scheme, tag, mesh in ((0, "firstorder", "m1d_s3_100"), (1, "weno3", "m1d_s5_100"), (2, "weno5", "m1d_s7_100")):
        gold = np.loadtxt(os.path.join(REF, f"tests_cpp/eigen_1d_euler_sod_explicit/{tag}/gold.txt"))
        h, s = ref.create(mesh, E1, 1, scheme, 1, {})
        U = np.empty(s[2])
        ref.L.ref_ic(h, vp(U))
        ref.L.ref_rk4(h, vp(U), 0.0, 1e-3, 100)
        ref.L.ref_destroy(h)
        assert np.allclose(U, gold, rtol=1e-9, atol=1e-11), ("sod", tag)
        traj[f"sod_{tag}"] = dict(mesh=mesh, family=E1, problem=1, scheme=scheme, icflag=1, stepper="rk4",
                                  dt=1e-3, steps=100, rtol=1e-9, atol=1e-11)
        np.save(os.path.join(GOLD, f"sod_{tag}.npy"), gold)
    # Riemann IC2: SSPRK3 dt=0.01 for StepCount(0.6/dt) steps, observer every 10 steps
    # (tests_cpp/eigen_2d_euler_riemann_explicit/main.cc:18-30, compare.py:43-55)
    nsteps = int(0.6 / 0.01)
    saved = (nsteps // 10) * 10
    for scheme, tag, mesh in ((0, "firstorder", "m2d_s3_20"), (1, "weno3", "m2d_s7_20"), (2, "weno5", "m2d_s7_20")):
        rho_g = np.loadtxt(os.path.join(REF, f"tests_cpp/eigen_2d_euler_riemann_explicit/{tag}/rho_gold.txt"))
        p_g = np.loadtxt(os.path.join(REF, f"tests_cpp/eigen_2d_euler_riemann_explicit/{tag}/p_gold.txt"))
        h, s = ref.create(mesh, E2, 4, scheme, 2, {})
        U = np.empty(s[2])
        ref.L.ref_ic(h, vp(U))
        ref.L.ref_ssprk3(h, vp(U), 0.0, 0.01, saved)
        ref.L.ref_destroy(h)
        D = U.reshape(-1, 4)
        rho = D[:, 0]
        u, v = D[:, 1] / rho, D[:, 2] / rho
        p = ((5. + 2.) / 5. - 1.) * (D[:, 3] - rho * (u ** 2 + v ** 2) * 0.5)
        assert np.allclose(rho, rho_g, rtol=1e-10, atol=1e-12), ("riemann rho", tag)
        assert np.allclose(p, p_g, rtol=1e-10, atol=1e-12), ("riemann p", tag)
        traj[f"riemann_{tag}"] = dict(mesh=mesh, family=E2, problem=4, scheme=scheme, icflag=2, stepper="ssprk3",
                                      dt=0.01, steps=saved, rtol=1e-10, atol=1e-12)
        np.savez(os.path.join(GOLD, f"riemann_{tag}.npz"), rho=rho_g, p=p_g)
    # SWE slip wall: RK4 dt=0.01 for StepCount(2/dt) steps, observer every 10
    # (tests_cpp/eigen_2d_swe_slip_wall_explicit/main.cc, compare.py)
    nsteps = int(2. / 0.01)
    saved = (nsteps // 10) * 10
    for scheme, tag, mesh in ((0, "firstorder", "m2d_s3_25"), (1, "weno3", "m2d_s5_25"), (2, "weno5", "m2d_s7_25")):
        h_g = np.loadtxt(os.path.join(REF, f"tests_cpp/eigen_2d_swe_slip_wall_explicit/{tag}/h_gold.txt"))
        h, s = ref.create(mesh, SW, 0, scheme, 1, {})
        U = np.empty(s[2])
        ref.L.ref_ic(h, vp(U))
        ref.L.ref_rk4(h, vp(U), 0.0, 0.01, saved)
        ref.L.ref_destroy(h)
        hh = U.reshape(-1, 3)[:, 0]
        assert np.allclose(hh, h_g, rtol=1e-10, atol=1e-12), ("swe", tag)
        traj[f"swe_{tag}"] = dict(mesh=mesh, family=SW, problem=0, scheme=scheme, icflag=1, stepper="rk4",
                                  dt=0.01, steps=saved, rtol=1e-10, atol=1e-12)
        np.save(os.path.join(GOLD, f"swe_{tag}.npy"), h_g)
    # Cross shock (defaults 0.1, 10, 1) and double Mach reflection: SSPRK3
    # dt=1e-3, 100 and 150 steps, observer every 50 steps, density of the last
    # snapshot (tests_cpp/eigen_2d_euler_cross_shock_explicit/main.cc,
    # tests_cpp/eigen_2d_euler_double_mach_reflection_explicit/main.cc, compare.py)
    for base, prob, steps, tags in (("cross", 7, 100, ((0, "firstorder", 3), (1, "weno3", 5), (2, "weno5", 7))),
                                    ("dmr", 6, 150, ((0, "firstorder", 3), (1, "weno3", 5)))):
        d = "eigen_2d_euler_cross_shock_explicit" if base == "cross" else "eigen_2d_euler_double_mach_reflection_explicit"
        for scheme, tag, st in tags:
            mesh = f"m2d_s{st}_40x20_cross" if base == "cross" else f"m2d_s{st}_60x15_dmr"
            rho_g = np.loadtxt(os.path.join(REF, "tests_cpp", d, tag, "rho_gold.txt"))
            h, s = ref.create(mesh, E2, prob, scheme, 1, {})
            U = np.empty(s[2])
            ref.L.ref_ic(h, vp(U))
            ref.L.ref_ssprk3(h, vp(U), 0.0, 1e-3, steps)
            ref.L.ref_destroy(h)
            assert np.allclose(U.reshape(-1, 4)[:, 0], rho_g, rtol=1e-10, atol=1e-12), (base, tag)
            traj[f"{base}_{tag}"] = dict(mesh=mesh, family=E2, problem=prob, scheme=scheme, icflag=1,
                                         stepper="ssprk3", dt=1e-3, steps=steps, rtol=1e-10, atol=1e-12)
            np.save(os.path.join(GOLD, f"{base}_{tag}.npy"), rho_g)
    json.dump(traj, open(os.path.join(GOLD, "trajectories.json"), "w"), indent=1)

    # Golds on meshes the tests regenerate (too large to keep as fixtures):
    # * the reference's Python tests, advanced by the Python driver's own
    #   SSP-RK3 update (pressiodemoapps/__init__.py:155-185): cross shock 80x40
    #   first order, dt 1e-3, 1000 steps (tests_py/2d_euler_cross_shock); double
    #   Mach reflection 200x50 first order and WENO3, dt 5e-4, 500 steps
    #   (tests_py/2d_double_mach_reflection) -- density golds;
    # * 3D Sedov symmetry, SSP-RK3 dt 1e-4, 250 steps, on [0, 0.4]^3 with 20^3
    #   and 20x25x28 cells, first order and WENO3, whole-state golds at rtol
    #   1e-8 / atol 1e-10 (tests_cpp/eigen_3d_euler_sedov_symmetry, compare.py).
    gen = {}
    runs = [
        ("cross_py_firstorder", "tests_py/2d_euler_cross_shock/rho_gold.txt", E2, 7, 0, 3, (80, 40),
         (0.0, 2.0, 0.0, 1.0), "ssprk3_py", 1e-3, 1000, "rho", 1e-10, 1e-12),
        ("dmr_py_firstorder", "tests_py/2d_double_mach_reflection/firstorder/rho_gold.txt", E2, 6, 0, 3,
         (200, 50), (0.0, 4.0, 0.0, 1.0), "ssprk3_py", 5e-4, 500, "rho", 1e-10, 1e-12),
        ("dmr_py_weno3", "tests_py/2d_double_mach_reflection/weno3/rho_gold.txt", E2, 6, 1, 5, (200, 50),
         (0.0, 4.0, 0.0, 1.0), "ssprk3_py", 5e-4, 500, "rho", 1e-10, 1e-12),
    ]
    for tag, scheme, st in (("firstorder", 0, 3), ("weno3", 1, 5)):
        for shape, n in (("equal", (20, 20, 20)), ("not_equal", (20, 25, 28))):
            runs.append((f"sedov3d_{tag}_{shape}",
                         f"tests_cpp/eigen_3d_euler_sedov_symmetry/{tag}_nxnynz_{shape}/gold_state.txt", E3, 1,
                         scheme, st, n, (0.0, 0.4, 0.0, 0.4, 0.0, 0.4), "ssprk3", 1e-4, 250, "state", 1e-8,
                         1e-10))
    import tempfile
    for (name, gsrc, fam, prob, scheme, st, n, bounds, stepper, dt, steps, field, rtol, atol) in runs:
        gold = np.loadtxt(os.path.join(REF, gsrc))
        with tempfile.TemporaryDirectory() as tmp:
            nargs = " ".join(str(v) for v in n)
            bargs = " ".join(str(v) for v in bounds)
            run(f"{sys.executable} {REF}/meshing_scripts/create_full_mesh.py -n {nargs} --bounds {bargs} "
                f"-s {st} --outDir {tmp}")
            L = ref.L
            names = (C.c_char_p * 1)()
            vals = (C.c_double * 1)()
            h = L.ref_create(tmp.encode(), fam, prob, scheme, 1, 0, names, vals)
            assert h, L.ref_last_error()
        sz = (C.c_long * 4)()
        L.ref_sizes(h, sz)
        U = np.empty(sz[2])
        L.ref_ic(h, vp(U))
        if stepper == "ssprk3":
            L.ref_ssprk3(h, vp(U), 0.0, dt, steps)
        else:
            v = np.empty(sz[1])
            t = 0.0
            for _ in range(steps):
                L.ref_velocity(h, vp(U), t, vp(v))
                u1 = U + dt * v
                L.ref_velocity(h, vp(u1), t + dt, vp(v))
                u2 = 3. / 4. * U + 1. / 4. * u1 + 1. / 4. * dt * v
                L.ref_velocity(h, vp(u2), t + dt * 0.5, vp(v))
                U = 1. / 3. * (U + 2. * u2 + 2. * dt * v)
                t += dt
        L.ref_destroy(h)
        nd = sz[0]
        got = U.reshape(-1, nd)[:, 0] if field == "rho" else U
        assert np.allclose(got, gold, rtol=rtol, atol=atol), name
        gen[name] = dict(n=list(n), bounds=list(bounds), stencil=st, family=fam, problem=prob, scheme=scheme,
                         icflag=1, stepper=stepper, dt=dt, steps=steps, field=field, rtol=rtol, atol=atol)
        np.save(os.path.join(GOLD, name + ".npy"), gold)
        print("gold", name)
    json.dump(gen, open(os.path.join(GOLD, "trajectories_generated_mesh.json"), "w"), indent=1)

    # Crank-Nicolson + Newton + BiCGSTAB gold of the reference's implicit
    # Riemann test (first order, 20x20, dt 0.02, 30 steps, Newton tolerance 1e-5)
    src = os.path.join(REF, "tests_cpp/eigen_2d_euler_riemann_implicit/firstorder")
    np.save(os.path.join(GOLD, "riemann_implicit_fo_rho.npy"), np.loadtxt(os.path.join(src, "rho_gold.txt")))
    np.save(os.path.join(GOLD, "riemann_implicit_fo_p.npy"), np.loadtxt(os.path.join(src, "p_gold.txt")))
    # ... and of the implicit double Mach reflection test (first order, 60x15,
    # Crank-Nicolson dt 0.01, 100 steps, Newton tolerance 1e-5)
    src = os.path.join(REF, "tests_cpp/eigen_2d_euler_double_mach_reflection_implicit/firstorder")
    np.save(os.path.join(GOLD, "dmr_implicit_fo_rho.npy"), np.loadtxt(os.path.join(src, "rho_gold.txt")))

    # mesh-generator golds (tests_mesh/mesh_generation_full_{1,2,3}d/*/*_gold.dat),
    # with the generator arguments their test.cmake files pass
    mg = os.path.join(GOLD, "mesh_generation")
    os.makedirs(mg, exist_ok=True)
    args = {}
    bounds = {1: [0.0, 1.0], 2: [0.0, 1.0, 0.0, 1.0], 3: [0.0, 1.0, 0.0, 2.0, 0.0, 3.0]}
    for dim, dd in ((1, "mesh_generation_full_1d"), (2, "mesh_generation_full_2d"), (3, "mesh_generation_full_3d")):
        base = os.path.join(REF, "tests_mesh", dd)
        for sub in sorted(os.listdir(base)):
            src = os.path.join(base, sub)
            if not os.path.isdir(src):
                continue
            cm = open(os.path.join(src, "CMakeLists.txt")).read()
            val = lambda k, d=None: (re.search(r"-D%s=(\S+)" % k, cm).group(1).strip('"') if re.search(r"-D%s=" % k, cm) else d)
            n = [int(val("nx")), int(val("ny", 1)), int(val("nz", 1))]
            per = val("PER")
            if dim == 1:
                p3 = [per not in ("0", "none"), False, False]
            elif dim == 2:
                p3 = [per in ("all", "onlyx"), per in ("all", "onlyy"), False]
            else:
                p3 = [per not in ("0", "none")] * 3
            args[sub] = dict(dim=dim, n=n, stencil=int(val("ss")), periodic=p3, bounds=bounds[dim])
            dst = os.path.join(mg, sub)
            os.makedirs(dst, exist_ok=True)
            for f in ("info", "connectivity", "coordinates"):
                shutil.copy(os.path.join(src, f + "_gold.dat"), os.path.join(dst, f + ".dat"))
    json.dump(args, open(os.path.join(mg, "args.json"), "w"), indent=1)


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "include", "pressiodemoapps")):
        sys.exit("set PDA_REFERENCE to a pressio-demoapps checkout")
    make_meshes()
    ref = Ref()
    manifest = make_cases(ref)
    json.dump(manifest, open(os.path.join(HERE, "manifest.json"), "w"), indent=1)
    make_gold(ref)
    print("done")


if __name__ == "__main__":
    main()
