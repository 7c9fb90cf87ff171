"""The tensor-core BF16 GEMM (tcgen05, TMEM accumulator) against a plain PyTorch fp32 reference
of the same op: BF16 inputs are exact in fp32, so the only difference is the order of the fp32
accumulation (relative error well below 1e-5)."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(lib, a, b, splits=1):
    import torch

    m, k = a.shape
    n = b.shape[0]
    kt = k // 64
    per = -(-kt // splits)
    nz = -(-kt // per)
    d = torch.full((nz, m, n), float("nan"), device="cuda", dtype=torch.float32)
    st = torch.zeros(4, device="cuda", dtype=torch.int32)
    rc = lib.wg_gemm_bf16_dev(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                              ctypes.c_void_p(d.data_ptr()), m, n, k, splits, ctypes.c_void_p(st.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(st[0]) == 0
    return d


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (256, 64, 128), (300, 64, 576), (1000, 576, 64), (313, 4, 128),
                                   (4900, 64, 576)])
def test_gemm_matches_fp32_reference(cuda_lib, m, n, k):
    import torch

    g = torch.Generator(device="cuda").manual_seed(m * 7 + n + k)
    a = torch.randn((m, k), device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16)
    d = _gemm(cuda_lib, a, b)[0]
    ref = a.float() @ b.float().t()
    err = float((d - ref).abs().max() / ref.abs().max())
    assert err < 1e-5, err


def test_gemm_split_k_partials_sum_to_the_product(cuda_lib):
    import torch

    g = torch.Generator(device="cuda").manual_seed(3)
    m, n, k = 576, 64, 64 * 50
    a = torch.randn((m, k), device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16)
    d = _gemm(cuda_lib, a, b, splits=7)
    assert d.shape[0] == 7
    ref = a.float() @ b.float().t()
    err = float((d.sum(0) - ref).abs().max() / ref.abs().max())
    assert err < 1e-5, err
