"""tcgen05 BF16 GEMM (tensor memory accumulators) against a plain PyTorch
fp32 matmul of the same bf16 operands.

Tolerance: both sides accumulate in fp32 in different orders, so entries
agree to a few fp32 ulps of sum_k |a_ik b_jk| (bound 1e-5 of that sum); the
bf16 output agrees with the bf16 rounding of the reference to one bf16 ulp."""
from __future__ import annotations

import pytest

SHAPES = [(128, 128, 64), (256, 384, 128), (200, 130, 192), (256, 1024, 4096), (384, 256, 1024),
          (128, 256, 16384), (200, 100, 8192),  # the last two take the split-K path
          # N <= 16: the thin blocked GEMM of the ROM decoder's output layer (operands blocked by
          # 64-column slices, one bulk copy per slice); the last two split K
          (96, 12, 64), (1000, 13, 1024), (23916, 13, 1024), (300, 16, 4096), (2000, 1, 2048)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{m}x{n}x{k}" for m, n, k in SHAPES])
@pytest.mark.parametrize("epi", [0, 1, 2])
def test_tc_gemm_matches_torch_fp32(pda, shape, epi):
    import torch
    M, N, K = shape
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K + epi)
    A = (torch.randn(M, K, generator=g, device="cuda") * 0.5).to(torch.bfloat16)
    B = (torch.randn(N, K, generator=g, device="cuda") * 0.5).to(torch.bfloat16)
    bias = torch.randn(N, generator=g, device="cuda") if epi else None
    cf, cb, pa = pda.tc_gemm_bf16(A, B, bias, epi, out_f32=True, out_bf16=True, preact=True)
    ref = A.float() @ B.float().T
    if epi:
        ref = ref + bias[None, :]
    scale = A.float().abs() @ B.float().abs().T + 1.0
    assert ((pa - ref).abs() <= 1e-5 * scale).all(), float(((pa - ref).abs() / scale).max())
    act = torch.nn.functional.elu(ref) if epi == 2 else ref
    tol = 1e-5 * scale + (1e-6 if epi == 2 else 0.0)
    assert ((cf - act).abs() <= tol).all(), float(((cf - act).abs() / scale).max())
    # bf16 output: the rounding of the fp32 result
    assert ((cb.float() - act).abs() <= act.abs() * 2 ** -8 + tol).all()


@pytest.mark.gpu
def test_tc_gemm_rejects_bad_k(pda):
    import torch
    A = torch.zeros(128, 96, dtype=torch.bfloat16, device="cuda")
    with pytest.raises(pda.PdaError):
        pda.tc_gemm_bf16(A, A)
