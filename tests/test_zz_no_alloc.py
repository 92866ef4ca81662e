"""The allocation-free Gram entry point (ttg_gram_noalloc), called through the
C ABI by a caller that owns all device memory, against NumPy's X^T Y.

Callers such as memory-pool owners or plugins that may not call cudaMalloc
hand in their own device buffers; the entry point keeps its partial sums in a
fixed device array inside the library.  This file is collected last so that
a failure here cannot hide any other test."""
import ctypes

import numpy as np
import pytest

from ttdft_public_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_gram_noalloc_matches_numpy_on_two_calls_in_a_row(small_system):
    import torch

    s = small_system
    lib = _lib.ttg()
    rng = np.random.default_rng(31)
    for call, k in enumerate((40, 24)):
        X = rng.standard_normal((s.N, k))
        Y = rng.standard_normal((s.N, k))
        ref = X.T @ Y
        # caller-owned device buffers: row-major n x k (ld = k) in, k x k column-major out
        xd = torch.from_numpy(np.ascontiguousarray(X)).cuda()
        yd = torch.from_numpy(np.ascontiguousarray(Y)).cuda()
        sd = torch.full((k, k), np.nan, dtype=torch.float64, device="cuda")
        rc = lib.ttg_gram_noalloc(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()),
                                  s.N, k, k, ctypes.c_void_p(sd.data_ptr()), None)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        got = sd.cpu().numpy().T            # column-major k x k
        # the Gram parity test's tolerance: 1e-13 of the largest entry
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max(), f"call {call}"


def test_gram_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    lib = _lib.ttg()
    x = torch.zeros(16, 8, dtype=torch.float64, device="cuda")
    s = torch.zeros(8, 8, dtype=torch.float64, device="cuda")
    k = 1449                                   # 1449^2 > 2,097,152 scratch doubles
    rc = lib.ttg_gram_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()), 16, k,
                              k, ctypes.c_void_p(s.data_ptr()), None)
    assert rc == 1                             # TTG_BAD_ARG, nothing launched
