"""pda::div_const (Markstein's correction step for a division by a constant,
used for the /3 and /6 of the WENO5 gradients) equals IEEE division bit for
bit on 8.8 million arguments (random over a wide exponent range, both signs,
exact multiples).  Host build of the same header the kernels use; the device
kernels are in turn checked bit for bit against the oracle's divisions by the
GPU parity tests."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pressio-demoapps_gb300", "csrc")


def test_div_const_matches_ieee_division(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "div_const_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC, "-o", exe,
                    os.path.join(HERE, "div_const_check.cpp"), "-lm"], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    bad, n = int(out[0]), int(out[1])
    assert n > 8_000_000
    assert bad == 0, f"{bad} of {n} quotients differ from IEEE division"
