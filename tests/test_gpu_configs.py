"""GPU parity at the benchmark's own sizes (not toy systems).

Configuration 1 (8 atoms, N = 8,000, 16 states, degree 20, fixed potential):
the plain FP64 Chebyshev-filtered subspace iteration runs on the GPU until
the residual ||H x_i - lambda_i x_i|| of every occupied state (N_e / 2 = 12)
is below 1e-8, and those eigenvalues must match ARPACK's (scipy) within
1e-6 Ha; its first two passes must match the oracle's passes from the same
start block and bounds.  The residual bound applies to the occupied states:
with the reference's bounds the filter's lower cut is the block's largest
Ritz value, so the top states of the block converge arbitrarily slowly (the
16th not at all).

Configuration 2 (64 atoms, N = 64,000, 160 states, degree 30, nonlocal
projectors): one FP64 pass against the oracle's pass on the same start
block and bounds; then the mixed-precision path and the FP64 schedule are
each run to convergence, and their occupied eigenvalues must agree within
1e-6 Ha and their densities (Fermi-Dirac occupations at 500 K) within the
bound stated in the test.  The mixed path is the one the SCF takes: the
BF16 schedule (BF16 first quarter of the degrees, FP32 after) while the
eigenvalues still move, then FP32 degrees only.  BF16 degrees alone stall:
the BF16 rounding they inject (2^-9 of the block) is damped only by the
degrees after them, which leaves residuals ~1e-3 on the highest occupied
states.

Configuration 3 (Hartree kernel expansion, core 60^3, 360 points per
direction, 35 terms) against the FP64 oracle.

Passes follow the restart and bound logic of main.cc:977-1207: the first pass
filters [0, upper] with a0 from Lanczos, later passes [w_max, upper] with
a0 = w_min of the previous Rayleigh-Ritz step.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

import oracle
from ttdft_public_gb300 import api, system
from ttdft_public_gb300.scf import KB_HA_PER_K

pytestmark = pytest.mark.gpu


def lanczos(op, n, seed=0):
    v0 = np.random.default_rng(seed).uniform(0.0, 1.0, n)
    return api.EigenSolver(op).computeUpperBoundWithLanczos(None, 20, v0=v0)


def residuals(op, X, w):
    """||H x_i - w_i x_i|| for the columns of the device block X (FP64)."""
    ax = api.AX(1, X.k)
    ax.op = op
    HX = api.Mat(op, X.k)
    ax.perform_ax(X, HX)
    Xh, HXh = X.get(), HX.get()
    HX.close()
    return np.linalg.norm(HXh - Xh * w[None, :], axis=0)


def run_passes(op, X, m, upper, lower, sch, max_passes, stop=None):
    """ChFSI passes with the reference's bound updates; stop(w) ends early."""
    a, a0 = 0.0, lower
    w = None
    for p in range(max_passes):
        w = api.chfsi_pass(op, X, m, a, upper, a0, sch, rotate=True)
        a0, a = w[0], w[-1]
        if stop is not None and stop(w, p):
            return w, p + 1
    return w, max_passes


def test_config1_fp64_chfsi_to_residual_1e8_matches_exact_eigenvalues(atoms8_system):
    s = atoms8_system
    k, m = s.spec.n_states, s.spec.degree
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), k)
    upper, lower = lanczos(op, s.N)
    X0 = np.random.default_rng(8).standard_normal((s.N, k))
    sch = api.sched("fp64", return_prev=True)   # the reference's filter (degree m-1 result)

    # the first two passes against the oracle's, same start block and bounds
    X = api.Mat(op, k, X0)
    w2, _ = run_passes(op, X, m, upper, lower, sch, 2)
    Xr, a, a0 = X0, 0.0, lower
    for _ in range(2):
        wr, _, Xr = oracle.chfsi_pass(s, Xr, m, a, upper, a0, return_prev=True)
        a0, a = wr[0], wr[-1]
    assert np.abs(w2 - wr).max() < 1e-9 * np.abs(wr).max()

    # to convergence: the residual of every occupied state below 1e-8
    n_occ = s.spec.n_electrons // 2
    res_hist = []

    def converged(w, p):
        r = residuals(op, X, w)
        res_hist.append(float(r[:n_occ].max()))
        return res_hist[-1] < 1e-8

    w, n_pass = run_passes(op, X, m, upper, lower, sch, 200, stop=converged)
    assert res_hist[-1] < 1e-8, f"residual {res_hist[-1]:.2e} after {n_pass} passes"
    exact = np.sort(sla.eigsh(s.H.to_scipy(), k=k, which="SA", tol=1e-13, ncv=64,
                              v0=np.ones(s.N), return_eigenvectors=False))
    assert np.abs(w[:n_occ] - exact[:n_occ]).max() < 1e-6
    op.close()


@pytest.fixture(scope="module")
def atoms64_system():
    return system.build_system(system.CONFIGS["atoms64"])


def test_config2_fp64_pass_matches_oracle_and_mixed_converges_to_fp64(atoms64_system):
    s = atoms64_system
    k, m = s.spec.n_states, s.spec.degree
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), k)
    upper, lower = lanczos(op, s.N)
    X0 = np.random.default_rng(64).standard_normal((s.N, k))

    # one plain FP64 pass against the oracle's
    X = api.Mat(op, k, X0)
    w1 = api.chfsi_pass(op, X, m, 0.0, upper, lower, api.sched("fp64"), rotate=True)
    wr, _, _ = oracle.chfsi_pass(s, X0, m, 0.0, upper, lower)
    assert np.abs(w1 - wr).max() < 1e-9 * np.abs(wr).max()
    X.close()

    # mixed (BF16 schedule, then FP32 degrees only) and FP64, each to
    # convergence of the occupied states (N_e/2 + 10, main.cc:686-688)
    n_occ = min(int(s.spec.n_electrons / 2 + 10), k - 1)
    runs = {}
    mixed = api.sched("fp32", low="bf16", n_low=m // 4)
    for name, stages in (("mixed", ((mixed, 1e-6), (api.sched("fp32"), 1e-10))),
                         ("fp64", ((api.sched("fp64"), 1e-10),))):
        Xm = api.Mat(op, k, X0)
        a, a0, w, n_pass = 0.0, lower, None, 0
        for sch, tol in stages:
            prev = None
            for _ in range(40):
                w = api.chfsi_pass(op, Xm, m, a, upper, a0, sch, rotate=True)
                a0, a = w[0], w[-1]
                n_pass += 1
                if prev is not None and np.abs(w[:n_occ] - prev[:n_occ]).max() < tol:
                    break
                prev = w.copy()
        runs[name] = (w, Xm, residuals(op, Xm, w), n_pass)
    wm, Xmix, rm, pm = runs["mixed"]
    wf, Xf, rf, pf = runs["fp64"]
    dw = np.abs(wm[:n_occ] - wf[:n_occ]).max()
    print(f"config 2: passes mixed {pm}, fp64 {pf}; max residual mixed {rm[:n_occ].max():.2e}, "
          f"fp64 {rf[:n_occ].max():.2e}; max |dlambda| {dw:.2e} Ha")
    assert rf[:n_occ].max() < 1e-6 and rm[:n_occ].max() < 1e-4
    assert dw < 1e-6
    # densities of the two converged subspaces with the SCF's occupations
    kT = KB_HA_PER_K * 500.0
    _, occ_m = api.fermi(op, wm, s.spec.n_electrons, kT)
    _, occ_f = api.fermi(op, wf, s.spec.n_electrons, kT)
    dm = api.density(op, Xmix, occ_m, s.basis)
    df = api.density(op, Xf, occ_f, s.basis)
    drho = np.linalg.norm(dm - df) / np.linalg.norm(df)
    print(f"config 2: density rel L2 {drho:.2e}")
    assert drho < 2e-5
    op.close()


def config3_case(rank=60):
    """Configuration 3: core 60^3, 360 quadrature points per direction of the
    32-bohr, 120-element mesh, 64 seeded Gaussian charge blobs, 35 terms."""
    return system.hartree_blob_case(rank=rank)


def test_config3_hartree_35_terms_against_fp64():
    alpha, omega, G, quad, U, grids = config3_case()
    assert G.shape == (60, 60, 60) and U[0].shape == (360, 60) and alpha.size == 35
    V, ms = api.hartree(alpha, omega, G, quad, U, grids)
    ref = oracle.hartree(alpha, omega, G, quad, U, grids)
    err = np.linalg.norm(V - ref) / np.linalg.norm(ref)
    print(f"config 3 Hartree: rel L2 {err:.3e}, contractions {ms:.3f} ms")
    assert err <= 1e-7
