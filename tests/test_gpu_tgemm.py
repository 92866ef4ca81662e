"""The tensor-core contraction engine (ttg_tc_gemm, the kernel behind the
Hartree and density contractions) against exact and FP64 products.

Integer-valued operands whose slices are the values themselves must come out
exact: every level sum is an integer below 2^24, which the tensor-memory
accumulators hold without rounding.  Random FP32 operands carry their FP32
quantisation on the slicing grid (2^-25 of each group's largest value)."""
import ctypes

import numpy as np
import pytest

from ttdft_public_gb300 import _lib

pytestmark = pytest.mark.gpu


def tc_gemm(A, B, groups):
    import torch
    m, k = A.shape
    n = B.shape[0]
    a = torch.from_numpy(np.ascontiguousarray(A, np.float32)).cuda()
    b = torch.from_numpy(np.ascontiguousarray(B, np.float32)).cuda()
    c = torch.full((m, n), np.nan, dtype=torch.float64, device="cuda")
    rc = _lib.ttg().ttg_tc_gemm(m, n, k, ctypes.c_void_p(a.data_ptr()), k,
                                ctypes.c_void_p(b.data_ptr()), k, groups,
                                ctypes.c_void_p(c.data_ptr()), n, None)
    assert rc == 0, rc
    return c.cpu().numpy()


@pytest.mark.parametrize("k", [64, 192])
def test_integer_operands_are_exact(k):
    rng = np.random.default_rng(k)
    A = rng.integers(-255, 256, (300, k)).astype(np.float32)
    B = rng.integers(-255, 256, (200, k)).astype(np.float32)
    C = tc_gemm(A, B, 1)
    assert np.array_equal(C, A.astype(np.float64) @ B.astype(np.float64).T)


def test_random_operands_grouped_against_fp64():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((300, 2240)).astype(np.float32)
    B = rng.standard_normal((200, 2240)).astype(np.float32)
    C = tc_gemm(A, B, 35)
    X = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    assert (np.abs(C - X) / scale).max() < 2e-7
