"""The CUDA path against the committed golden fixtures (tests/golden/tiny.npz),
through the C ABI.  Tolerances as in the parity tests: FP64 paths to
summation order, eigenvalues to 1e-8 Ha after the same six passes, SCF
energies per iteration to 3e-5 Ha (FP32 Hartree potential on the GPU)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden as mg  # noqa: E402

from ttdft_public_gb300 import _lib, api, scf, system  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    return np.load(mg.OUT)


@pytest.fixture(scope="module")
def tiny():
    return system.build_system(system.small_spec())


def test_filter_lanczos_and_chfsi_against_fixtures(gold, tiny):
    s = tiny
    k = s.spec.n_states
    X0, v0 = mg.inputs(s)
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), k)
    try:
        ax = api.AX(1, k)
        ax.op = op
        f = mg.FILTER
        for key, prev in (("filter_prev", True), ("filter_m", False)):
            Xm = api.Mat(op, k, X0)
            api.ChebyShevFilter(api.sched("fp64", return_prev=prev)).computeFilteredSubspace(
                None, ax, Xm, s.N, f["m"], f["a"], f["b"], f["a0"])
            ref = gold[key]
            assert np.abs(Xm.get() - ref).max() < 1e-11 * np.abs(ref).max()
        up, lo = api.EigenSolver(op).computeUpperBoundWithLanczos(None, mg.LANCZOS_ITERS, v0=v0)
        rup, rlo = gold["lanczos_bounds"]
        assert abs(up - rup) < 1e-9 * abs(rup) and abs(lo - rlo) < 1e-9 * max(1.0, abs(rlo))
        Xm = api.Mat(op, k, X0)
        a, a0 = 0.0, lo
        for _ in range(mg.PASSES):
            w = api.chfsi_pass(op, Xm, s.spec.degree, a, up, a0, api.sched("fp64"), rotate=True)
            a0, a = w[0], w[-1]
        assert np.abs(w - gold["chfsi_eigenvalues"]).max() < 1e-8
    finally:
        op.close()


def test_lda_and_scf_against_fixtures(gold):
    import torch
    rho = torch.from_numpy(gold["lda_rho"].copy()).cuda()
    v = torch.zeros_like(rho)
    e = torch.zeros_like(rho)
    assert _lib.ttg().ttg_grid_lda(rho.data_ptr(), rho.numel(), v.data_ptr(), e.data_ptr(), 0,
                                   None) == 0
    assert np.allclose(v.cpu().numpy(), gold["lda_v"], rtol=1e-12)
    assert np.allclose(e.cpu().numpy(), gold["lda_e"], rtol=1e-12)
    run = scf.Scf(system.build_system(mg.scf_spec()), mg.scf_config()).run()
    eg = np.array([h["energy"] for h in run["history"]])
    assert eg.shape == gold["scf_energies"].shape
    assert np.abs(eg - gold["scf_energies"]).max() < 3e-5
