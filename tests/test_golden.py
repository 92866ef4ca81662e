"""The oracle against the committed golden fixtures (tests/golden/tiny.npz,
written by tests/golden/make_golden.py): a regression anchor for the
checker itself, on the same seeded systems the GPU tests use."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden as mg  # noqa: E402

import oracle  # noqa: E402
from oracle import scf as oscf  # noqa: E402
from ttdft_public_gb300 import system  # noqa: E402


@pytest.fixture(scope="module")
def gold():
    return np.load(mg.OUT)


@pytest.fixture(scope="module")
def tiny():
    return system.build_system(system.small_spec())


def test_system_generator_unchanged(gold, tiny):
    s = tiny
    fp = np.array([s.N, s.H.row_ptr[-1], s.H.val.sum(), np.abs(s.C.val).sum()])
    assert np.allclose(fp, gold["fingerprint"], rtol=1e-12, atol=0)


def test_filter_and_lanczos(gold, tiny):
    X0, v0 = mg.inputs(tiny)
    f = mg.FILTER
    for key, prev in (("filter_prev", True), ("filter_m", False)):
        Y = oracle.cheb_filter(tiny, X0, f["m"], f["a"], f["b"], f["a0"], return_prev=prev)
        assert np.abs(Y - gold[key]).max() < 1e-12 * np.abs(gold[key]).max()
    al, be = oracle.lanczos_T(tiny, v0, mg.LANCZOS_ITERS)
    assert np.allclose(al, gold["lanczos_alpha"], rtol=1e-12, atol=1e-14)
    assert np.allclose(be, gold["lanczos_beta"], rtol=1e-12, atol=1e-14)


def test_chfsi_eigenvalues_and_lda(gold, tiny):
    X0, v0 = mg.inputs(tiny)
    up, lo = oracle.lanczos_bounds(tiny, v0, mg.LANCZOS_ITERS)
    X, a, a0 = X0, 0.0, lo
    for _ in range(mg.PASSES):
        w, _, X = oracle.chfsi_pass(tiny, X, tiny.spec.degree, a, up, a0)
        a0, a = w[0], w[-1]
    assert np.abs(w - gold["chfsi_eigenvalues"]).max() < 1e-10
    v, e = oscf.lda(gold["lda_rho"])
    assert np.allclose(v, gold["lda_v"], rtol=1e-14) and np.allclose(e, gold["lda_e"], rtol=1e-14)


def test_scf_energies(gold):
    run = oscf.OracleScf(system.build_system(mg.scf_spec()), mg.scf_config()).run()
    e = np.array([h["energy"] for h in run["history"]])
    assert e.shape == gold["scf_energies"].shape
    assert np.abs(e - gold["scf_energies"]).max() < 1e-9
