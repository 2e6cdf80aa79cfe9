"""The integer-pipe division and square root (csrc/fp64_intpipe.cuh), which
replace every FP64 division and square root of the residual kernels, return
the IEEE round-to-nearest results bit for bit: billions of seeded operand
sets per call, compared on the device with the FP64 pipe's operations
(pda_check_divsqrt), covering normal-range operands, divisor mantissas at
both ends of [1, 2), near-exact quotients and roots (rounding midpoints), and
arbitrary bit patterns (zeros, subnormals, infinities and NaNs take the
ordinary operations)."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_integer_pipe_division_and_sqrt_are_ieee(pda, mode):
    n, bad_div, bad_sqrt = pda.check_divsqrt(mode, seed=20261203 + mode, per_thread=2048)
    assert n >= 152 * 2048 * 2048 // 2
    assert bad_div == 0 and bad_sqrt == 0, (n, bad_div, bad_sqrt)


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_integer_pipe_exact_products_are_ieee(pda, mode):
    """The integer-pipe forms of K x (K = 3, 5, 7, 11, 13), x / 2, x / 4,
    x c for literal constants c and x + 1e-30, which replace those FP64
    operations in the residual kernels, equal the FP64 pipe's results bit for
    bit (ties, edges of the fast paths, zeros, subnormals, infinities and NaNs
    included)."""
    n, bad_k, bad_p2, bad_es, bad_c = pda.check_products(mode, seed=20261204 + mode, per_thread=2048)
    assert n >= 152 * 2048 * 2048 // 2
    assert bad_k == 0 and bad_p2 == 0 and bad_es == 0 and bad_c == 0, (n, bad_k, bad_p2, bad_es, bad_c)
