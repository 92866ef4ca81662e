"""The FP64 GEMMs on the tensor cores (ozgemm.cu: six exact BF16 digits per
value on per-row power-of-two scales, exact level sums in tensor memory,
double-FP32 across groups) against products computed in extended precision.
They serve the Gram matrices of Cholesky-QR and Rayleigh-Ritz and the block
products X L^-T and X Q; ttg_gram exposes the general X^T Y."""
import ctypes

import numpy as np
import pytest

import oracle
from ttdft_public_gb300 import _lib, api

pytestmark = pytest.mark.gpu


def exact_gram(X, Y):
    return (X.astype(np.longdouble).T @ Y.astype(np.longdouble)).astype(np.float64)


@pytest.mark.parametrize("k", [40, 96, 130])
def test_gram_matches_extended_precision(small_system, k):
    """Columns spread over 12 decades and rows over 6 (the filtered blocks'
    shape): every entry within 2^-44 of sum |x| |y| (the double-FP32 CUDA-core
    kernel this path replaces reaches about 2^-47 on short sums)."""
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(small_system), k)
    try:
        rng = np.random.default_rng(k)
        n = small_system.N
        X = rng.standard_normal((n, k)) * np.geomspace(1.0, 1e-12, k)
        X *= np.geomspace(1.0, 1e-6, n)[:, None]
        Y = rng.standard_normal((n, k)) * np.geomspace(1e3, 1e-3, k)
        S = api.MultTM().mult(api.Mat(op, k, X), api.Mat(op, k, Y))
        ref = exact_gram(X, Y)
        scale = np.abs(X).T @ np.abs(Y)
        assert np.max(np.abs(S - ref) / scale) < 2.0 ** -44
    finally:
        op.close()


def test_integer_blocks_are_exact(small_system):
    """Small integers are exact digits: X^T Y comes out exact."""
    k = 64
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(small_system), k)
    try:
        rng = np.random.default_rng(2)
        n = small_system.N
        X = rng.integers(-1000, 1001, (n, k)).astype(np.float64)
        Y = rng.integers(-1000, 1001, (n, k)).astype(np.float64)
        S = api.MultTM().mult(api.Mat(op, k, X), api.Mat(op, k, Y))
        assert np.array_equal(S, X.T @ Y)
    finally:
        op.close()


@pytest.mark.parametrize("k", [64, 200])
def test_rotation_and_orthonormalisation(small_system, k):
    """X Q (the Rayleigh-Ritz rotation) and Cholesky-QR (X L^-T, with the
    triangular B operand) against the oracle's FP64 restatement."""
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(small_system), k)
    try:
        rng = np.random.default_rng(7 + k)
        n = small_system.N
        X = rng.standard_normal((n, k)) * np.geomspace(1.0, 1e-4, k)
        Q, _ = np.linalg.qr(rng.standard_normal((k, k)))
        Xm = api.Mat(op, k, X)
        lib = _lib.ttg()
        Qf = np.asfortranarray(Q)
        assert lib.ttg_rotate(op.h, Xm.h, ctypes.c_void_p(Qf.ctypes.data)) == 0
        got = Xm.get()
        ref = oracle.rotate(X, Q)
        assert np.max(np.abs(got - ref)) < 2.0 ** -44 * np.max(np.abs(X) @ np.abs(Q))
        Xm = api.Mat(op, k, X)
        api.MultTM().orth(Xm)
        Qo = Xm.get()
        ref, st = oracle.cholqr(X)
        assert st == 0
        assert np.max(np.abs(Qo - ref)) < 1e-10
        # one Cholesky-QR of a block of condition ~1e4: orthogonality to
        # ~cond^2 u (FP64 gives the same order)
        assert np.abs(Qo.T @ Qo - np.eye(k)).max() < 1e-9
    finally:
        op.close()
