"""Build recipe for the CUDA shared library libpda_gb300.so (sm_103a only).

Every translation unit is compiled by nvcc in parallel, then linked into
``pressio-demoapps_gb300/lib/libpda_gb300.so`` (in-tree).  Floating-point
contraction is disabled on device (``-fmad=false``) and host
(``-ffp-contract=off``) so that results reproduce the reference's
double-precision operation order bit for bit.  The reduced-order-model units
(LSPG, GEMM launchers, autoencoder) owe the reference no bitwise parity and
are built with contraction on (``-fmad=true``); their tests bound them by
tolerances.

Usage: ``python pressio-demoapps_gb300/build_lib.py [--force] [--ptxas-verbose]``
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILDDIR = os.path.join(HERE, "_build")
LIBNAME = "libpda_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = [
    "kernels_euler2d.cu",
    "kernels_swe2d.cu",
    "kernels_euler3d.cu",
    "kernels_euler1d.cu",
    "util.cu",
    "noalloc.cu",
    "mlp.cu",
    "rom.cu",
    "ae.cu",
    "implicit.cu",
    "mesh.cpp",
    "problem.cpp",
    "batch.cpp",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


# translation units without a bitwise-parity obligation: FMA contraction on
CONTRACTED = {"rom.cu", "mlp.cu", "ae.cu"}


def _flags(ptxas_verbose: bool, src: str = "") -> list[str]:
    fmad = "-fmad=true" if src in CONTRACTED else "-fmad=false"
    f = ["-O3", "-std=c++17", "-lineinfo", fmad, "--expt-relaxed-constexpr",
         "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + CSRC]
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    return f + ARCH


def _needs_build(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, ptxas_verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILDDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "pda_gb300.h"))
    cc = nvcc()
    objs = []
    cmds = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(BUILDDIR, src + ".o")
        objs.append(obj)
        if force or _needs_build(obj, [sp] + headers):
            cmds.append([cc, *_flags(ptxas_verbose, src), "-c", sp, "-o", obj])

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p.returncode, p.stdout + p.stderr

    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            results = list(ex.map(run, cmds))
        failed = [r for r in results if r[1] != 0]
        for cmd, rc, out in results:
            if ptxas_verbose or rc != 0:
                sys.stderr.write(out)
        if failed:
            raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(c[0][-3]) for c in failed))
    out = lib_path()
    if force or cmds or _needs_build(out, objs):
        link = [cc, "-shared", *ARCH, "-o", out, *objs]
        p = subprocess.run(link, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, ptxas_verbose=a.ptxas_verbose))
