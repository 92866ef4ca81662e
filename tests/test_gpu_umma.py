"""The tcgen05 (tensor-memory) FP32 filter degree against the FP64 oracle and
against the mma.sync tensor-core kernel.  The kernel runs for block widths
that are multiples of 16 up to 256, wider blocks (288 here) in column blocks
of at most 256.  Its three-term BF16 split keeps FP32
accuracy, so the FP32 bound of the other FP32 kernels (5e-5 of the block's
largest entry after a 10-degree filter) applies; the kernel's own error is
reported by the tests as well."""
import numpy as np
import pytest

import oracle
from ttdft_public_gb300 import api, scf, system

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def run_filter(op, s, X, m, a, b, a0, prec="fp32"):
    k = X.shape[1]
    ax = api.AX(1, k)
    ax.op = op
    Xm = api.Mat(op, k, X)
    api.ChebyShevFilter(api.sched(prec)).computeFilteredSubspace(None, ax, Xm, s.N, m, a, b, a0)
    op.sync()
    return Xm.get()


def bounds(s, v_seed=6):
    v0 = np.random.default_rng(v_seed).uniform(0, 1, s.N)
    up, lo = oracle.lanczos_bounds(s, v0, 20)
    return 0.0, up, lo


@pytest.mark.parametrize("k", [16, 48, 160, 288])
@pytest.mark.parametrize("tucker", [True, False])
def test_umma_filter_matches_oracle(small_system, k, tucker):
    s = small_system
    H = api.ProjectHamiltonianSparse.from_system(s)
    if not tucker:
        H.ranks = None
    op = api.Operator(H, k)
    try:
        assert op.info()["umma_tiles"] > 0
        a, b, a0 = bounds(s)
        X = np.random.default_rng(20 + k).standard_normal((s.N, k))
        Y = run_filter(op, s, X, 10, a, b, a0)
        ref = oracle.cheb_filter(s, X, 10, a, b, a0)
        err = rel(Y, ref)
        print(f"k={k} tucker={tucker}: max error / max entry = {err:.2e}")
        assert err < 5e-5
    finally:
        op.close()


def test_umma_and_mma_sync_kernels_agree(small_system, monkeypatch):
    s = small_system
    k = 32
    a, b, a0 = bounds(s)
    X = np.random.default_rng(3).standard_normal((s.N, k))
    out = {}
    for name, disable in (("umma", "0"), ("mma_sync", "1")):
        monkeypatch.setenv("TTG_DISABLE_UMMA", disable)
        op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), k)
        try:
            assert (op.info()["umma_tiles"] > 0) == (disable == "0")
            out[name] = run_filter(op, s, X, 8, a, b, a0)
        finally:
            op.close()
    assert rel(out["umma"], out["mma_sync"]) < 5e-5


def test_umma_bf16_degrees_agree_with_mma_sync(small_system, monkeypatch):
    """BF16 degrees on tcgen05 (H rounded to BF16, one product per chunk)
    against the mma.sync BF16 kernel and the FP64 oracle.  Both round H and
    the block to BF16 and accumulate in FP32; they differ in summation order
    only, so they agree far more closely than either agrees with FP64."""
    s = small_system
    k = 32
    a, b, a0 = bounds(s)
    X = np.random.default_rng(4).standard_normal((s.N, k))
    out = {}
    for name, disable in (("umma", "0"), ("mma_sync", "1")):
        monkeypatch.setenv("TTG_DISABLE_UMMA", disable)
        op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), k)
        try:
            op.kernel_timing(True)
            out[name] = run_filter(op, s, X, 6, a, b, a0, prec="bf16")
            kind = "umma_bf16" if disable == "0" else "tc_bf16"
            assert op.kernel_time(kind)[1] == 6        # every degree on the expected kernel
        finally:
            op.close()
    ref = oracle.cheb_filter(s, X, 6, a, b, a0)
    e_umma, e_tc = rel(out["umma"], ref), rel(out["umma"], out["mma_sync"])
    print(f"bf16 degrees: tcgen05 vs FP64 {e_umma:.2e}, tcgen05 vs mma.sync {e_tc:.2e}")
    assert e_umma < 5e-2
    assert e_tc < 1e-2


def test_umma_filter_after_potential_update():
    """New H values written by the device update (all formats, the tcgen05
    planes included) against the oracle's Hamiltonian for the same V_eff."""
    from oracle import scf as oscf
    spec = system.small_spec(name="scf", n_atoms=2, box=10.0, n_el=16, rank=8, n_states=16,
                             degree=12, seed=3)
    s = system.build_system(spec)
    g = scf.Scf(s, scf.ScfConfig())
    c = oscf.OracleScf(s, scf.ScfConfig())
    try:
        veff = c.veff_from(c.initial_density())
        g.update_hamiltonian(g._dev(veff.reshape(-1)))
        assert g.op.info()["umma_tiles"] > 0

        class Sys:
            pass
        sh = Sys()
        sh.H, sh.C, sh.D, sh.N = c.hamiltonian(veff), s.C, s.D, s.N
        k = 16
        a, b, a0 = 0.0, 40.0, -1.0
        X = np.random.default_rng(8).standard_normal((s.N, k))
        Y = run_filter(g.op, s, X, 8, a, b, a0)
        ref = oracle.cheb_filter(sh, X, 8, a, b, a0)
        assert rel(Y, ref) < 5e-5
    finally:
        g.close()


def test_umma_bf16_degree_in_column_blocks(small_system):
    """A 288-wide block takes two tcgen05 launches per BF16 degree (144 + 144
    columns); each column's result matches the one a narrow block gives (to
    the BF16 rounding of the result) and the oracle's."""
    s = small_system
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), 288)
    try:
        a, b, a0 = bounds(s)
        X = np.random.default_rng(77).standard_normal((s.N, 288))
        Y = run_filter(op, s, X, 1, a, b, a0, prec="bf16")
        Y48 = run_filter(op, s, X[:, 144:192], 1, a, b, a0, prec="bf16")
        assert rel(Y[:, 144:192], Y48) < 1e-2
        ref = oracle.cheb_filter(s, X, 1, a, b, a0)
        assert rel(Y, ref) < 2e-2
    finally:
        op.close()
