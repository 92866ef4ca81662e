"""GPU parity: every libttg entry point against the FP64 oracle on the same
seeded inputs, through the C ABI.  Tolerances are stated per test:
  FP64 paths    ~1e-11 relative (summation order only)
  FP32 filter   5e-5 relative to the block's max entry (the tensor-core
                kernel's 3-term TF32 split keeps ~22 significant bits, so the
                12-degree recurrence loses a few more bits than FP32 FMAs)
  BF16 degrees  checked through the Ritz values they lead to
  eigenvalues   1e-6 Ha after convergence (the method's acceptance bound)
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
from ttdft_public_gb300 import api, system
from ttdft_public_gb300._lib import TtgError

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def dense_h(s):
    C = s.C.to_dense()
    return s.H.to_dense() + C.T @ np.diag(s.D) @ C


@pytest.fixture(scope="module")
def tiny_op(tiny_system):
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(tiny_system), 32)
    yield op
    op.close()


@pytest.fixture(scope="module")
def small_op(small_system):
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(small_system), 64)
    yield op
    op.close()


def bounds(s, k):
    w = np.linalg.eigvalsh(dense_h(s))
    return w, w[k + 4], w[-1] * 1.02, w[0]


def test_op_info_counts_nonzeros(tiny_op, tiny_system):
    inf = tiny_op.info()
    assert inf["n"] == tiny_system.N
    assert inf["nnz_h"] == tiny_system.H.nnz
    assert inf["nnz_c"] == tiny_system.C.nnz
    assert 0 < inf["fill"] <= 1.0


def test_block_roundtrip(tiny_op, tiny_system):
    X = np.random.default_rng(0).standard_normal((tiny_system.N, 7))
    B = api.Mat(tiny_op, 7, X)
    assert np.array_equal(B.get(), X)


@pytest.mark.parametrize("k", [1, 5, 16])
def test_apply_h_fp64(tiny_op, tiny_system, k):
    X = np.random.default_rng(k).standard_normal((tiny_system.N, k))
    ax = api.AX(1, k)
    ax.op = tiny_op
    Xm, Ym = api.Mat(tiny_op, k, X), api.Mat(tiny_op, k)
    ax.perform_ax(Xm, Ym)
    assert rel(Ym.get(), oracle.apply_h(tiny_system, X)) < 1e-12


@pytest.mark.parametrize("return_prev", [False, True])
@pytest.mark.parametrize("k", [6, 24])
def test_filter_fp64_matches_oracle(small_op, small_system, return_prev, k):
    s = small_system
    w, a, b, a0 = bounds(s, k)
    X = np.random.default_rng(10 + k).standard_normal((s.N, k))
    Xm = api.Mat(small_op, k, X)
    f = api.ChebyShevFilter(api.sched("fp64", return_prev=return_prev))
    ax = api.AX(1, k)
    ax.op = small_op
    f.computeFilteredSubspace(None, ax, Xm, s.N, 12, a, b, a0)
    ref = oracle.cheb_filter(s, X, 12, a, b, a0, return_prev=return_prev)
    assert rel(Xm.get(), ref) < 1e-11


@pytest.mark.parametrize("k", [8, 24, 36])
def test_filter_fp32_matches_oracle(small_op, small_system, k):
    s = small_system
    w, a, b, a0 = bounds(s, k)
    X = np.random.default_rng(20 + k).standard_normal((s.N, k))
    Xm = api.Mat(small_op, k, X)
    ax = api.AX(1, k)
    ax.op = small_op
    api.ChebyShevFilter(api.sched("fp32")).computeFilteredSubspace(None, ax, Xm, s.N, 12, a, b, a0)
    ref = oracle.cheb_filter(s, X, 12, a, b, a0)
    assert rel(Xm.get(), ref) < 5e-5


@pytest.mark.parametrize("k,ranks", [(40, True), (72, True), (200, True), (24, False)])
def test_filter_tensor_core_fp32_matches_oracle(small_system, k, ranks):
    """3-D tiled tensor-core SpMM (3xTF32): widths that are not multiples of
    32, more than one 160-state chunk (k=200), and the generic tiling used
    when the Tucker ranks are unknown."""
    s = small_system
    H = api.ProjectHamiltonianSparse.from_system(s)
    if not ranks:
        H.ranks = None
    op = api.Operator(H, 256)
    assert op.info()["n_tiles"] > 0
    w, a, b, a0 = bounds(s, 24)
    X = np.random.default_rng(40 + k).standard_normal((s.N, k))
    Xm = api.Mat(op, k, X)
    ax = api.AX(1, k)
    ax.op = op
    api.ChebyShevFilter(api.sched("fp32")).computeFilteredSubspace(None, ax, Xm, s.N, 10, a, b, a0)
    ref = oracle.cheb_filter(s, X, 10, a, b, a0)
    assert rel(Xm.get(), ref) < 5e-5
    op.close()


def test_filter_bf16_degree_matches_oracle(small_op, small_system):
    """One BF16 degree (H and the block rounded to BF16, FP32 accumulation):
    relative error of order the BF16 unit roundoff."""
    s = small_system
    w, a, b, a0 = bounds(s, 24)
    X = np.random.default_rng(50).standard_normal((s.N, 32))
    Xm = api.Mat(small_op, 32, X)
    ax = api.AX(1, 32)
    ax.op = small_op
    api.ChebyShevFilter(api.sched("bf16")).computeFilteredSubspace(None, ax, Xm, s.N, 1, a, b, a0)
    ref = oracle.cheb_filter(s, X, 1, a, b, a0)
    assert rel(Xm.get(), ref) < 2e-2


def test_tensor_core_and_cuda_core_kernels_agree(small_system, monkeypatch):
    s = small_system
    w, a, b, a0 = bounds(s, 24)
    X = np.random.default_rng(60).standard_normal((s.N, 48))
    out = {}
    for tc in ("0", "1"):
        monkeypatch.setenv("TTG_DISABLE_TC", "1" if tc == "0" else "0")
        op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), 48)
        assert (op.info()["n_tiles"] > 0) == (tc == "1")
        Xm = api.Mat(op, 48, X)
        ax = api.AX(1, 48)
        ax.op = op
        api.ChebyShevFilter(api.sched("fp32")).computeFilteredSubspace(None, ax, Xm, s.N, 8, a, b,
                                                                       a0)
        out[tc] = Xm.get()
        op.close()
    assert rel(out["1"], out["0"]) < 5e-5


def test_filter_degree_one_reference_returns_input(small_op, small_system):
    X = np.random.default_rng(3).standard_normal((small_system.N, 4))
    Xm = api.Mat(small_op, 4, X)
    ax = api.AX(1, 4)
    ax.op = small_op
    api.ChebyShevFilter(api.sched("fp64", return_prev=True)).computeFilteredSubspace(
        None, ax, Xm, small_system.N, 1, 0.5, 5.0, 0.1)
    assert np.array_equal(Xm.get(), X)


def test_gram_and_cholqr(small_op, small_system):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((small_system.N, 40))
    Y = rng.standard_normal((small_system.N, 40))
    Xm, Ym = api.Mat(small_op, 40, X), api.Mat(small_op, 40, Y)
    mt = api.MultTM()
    assert rel(mt.mult(Xm, Ym), X.T @ Y) < 1e-13
    mt.orth(Xm)
    Q = Xm.get()
    ref, st = oracle.cholqr(X)
    assert st == 0
    assert rel(Q, ref) < 1e-11
    assert np.abs(Q.T @ Q - np.eye(40)).max() < 1e-12


@pytest.mark.parametrize("k", [200, 329])
def test_blocked_cholqr_wide_blocks(small_system, k):
    """Blocks wider than 128 states take the blocked Cholesky (64-column
    panels on many CTAs, the inverse by block forward substitution): with
    column norms spread over 1e6 the result matches the oracle's Cholesky-QR,
    and a dependent column is still reported as NOT_SPD with X untouched."""
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(small_system), k)
    try:
        rng = np.random.default_rng(k)
        X = rng.standard_normal((small_system.N, k)) * np.geomspace(1.0, 1e-6, k)
        Xm = api.Mat(op, k, X)
        api.MultTM().orth(Xm)
        Q = Xm.get()
        ref, st = oracle.cholqr(X)
        assert st == 0
        assert rel(Q, ref) < 1e-9
        assert np.abs(Q.T @ Q - np.eye(k)).max() < 1e-10
        X[:, k - 5] = X[:, 150]
        Xm = api.Mat(op, k, X)
        with pytest.raises(TtgError) as e:
            api.MultTM().orth(Xm)
        assert e.value.status == "NOT_SPD"
        assert np.array_equal(Xm.get(), X)
    finally:
        op.close()


def test_cholqr_not_spd_is_reported_and_x_untouched(small_op, small_system):
    X = np.random.default_rng(5).standard_normal((small_system.N, 8))
    X[:, 6] = X[:, 2]
    Xm = api.Mat(small_op, 8, X)
    with pytest.raises(TtgError) as e:
        api.MultTM().orth(Xm)
    assert e.value.status == "NOT_SPD"
    assert np.array_equal(Xm.get(), X)


@pytest.mark.parametrize("k", [3, 20, 64, 161])
def test_syev_matches_lapack(k):
    s = system.build_system(system.small_spec())
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), 200)
    rng = np.random.default_rng(k)
    A = rng.standard_normal((k, k))
    A = A + A.T
    w = np.zeros(k)
    V = np.zeros((k, k), order="F")
    api.EigenSolver(op).computeEigenPairsSeq(A, k, k, w, V)
    wr, Vr = oracle.eigh(A)
    assert np.abs(w - wr).max() < 1e-12 * np.abs(wr).max()
    assert np.abs(np.abs(V.T @ Vr) - np.eye(k)).max() < 1e-9
    assert np.abs(A @ V - V * w).max() < 1e-11 * np.abs(wr).max()
    op.close()


def test_lanczos_bounds_match_oracle(small_op, small_system):
    v0 = np.random.default_rng(6).uniform(0, 1, small_system.N)
    up, lo = api.EigenSolver(small_op).computeUpperBoundWithLanczos(None, 20, v0=v0)
    rup, rlo = oracle.lanczos_bounds(small_system, v0, 20)
    assert abs(up - rup) < 1e-9 * abs(rup)
    assert abs(lo - rlo) < 1e-9 * max(1.0, abs(rlo))


def test_rayleigh_ritz_matches_oracle(small_op, small_system):
    s = small_system
    X, _ = oracle.cholqr(np.random.default_rng(7).standard_normal((s.N, 24)))
    Xm = api.Mat(small_op, 24, X)
    w = api.rayleigh_ritz(small_op, Xm, rotate=True)
    wr, Q, Xr = oracle.rayleigh_ritz(s, X)
    assert np.abs(w - wr).max() < 1e-11 * np.abs(wr).max()
    # rotated block: compare column by column up to sign
    Xg = Xm.get()
    dots = np.abs(np.sum(Xg * Xr, axis=0)) / (np.linalg.norm(Xg, axis=0) * np.linalg.norm(Xr, axis=0))
    assert np.all(dots > 1 - 1e-9)


def test_rayleigh_ritz_fp64_and_df64_agree(small_system):
    s = small_system
    X, _ = oracle.cholqr(np.random.default_rng(17).standard_normal((s.N, 40)))
    out = {}
    for prec in ("fp64", "df64"):
        op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), 40)
        op.set_rr_precision(prec)
        out[prec] = api.rayleigh_ritz(op, api.Mat(op, 40, X), rotate=False)
        op.close()
    wr, _, _ = oracle.rayleigh_ritz(s, X, rotate_x=False)
    # pairs of FP32 carry ~44 bits: Ritz values to ~1e-12 of the spectrum's scale
    assert np.abs(out["df64"] - wr).max() < 1e-11 * np.abs(wr).max()
    assert np.abs(out["fp64"] - wr).max() < 1e-11 * np.abs(wr).max()


def chfsi_converge(op, s, k, m, sch, passes, seed=8):
    """main.cc:987-1207 restart loop, GPU path."""
    v0 = np.random.default_rng(seed).uniform(0, 1, s.N)
    upper, lower = api.EigenSolver(op).computeUpperBoundWithLanczos(None, 20, v0=v0)
    X = np.random.default_rng(seed + 1).standard_normal((s.N, k))
    Xm = api.Mat(op, k, X)
    a, a0 = 0.0, lower
    w = None
    for _ in range(passes):
        w = api.chfsi_pass(op, Xm, m, a, upper, a0, sch, rotate=True)
        a0, a = w[0], w[-1]
    return w, Xm


@pytest.mark.parametrize("mode", ["fp64", "fp32", "mixed"])
def test_chfsi_converges_to_exact_eigenvalues(small_op, small_system, mode):
    # mixed: BF16 for the first quarter of the degrees, FP32 after (the
    # schedule of the large workloads).  Rounding made in a BF16 degree is
    # damped by the remaining FP32 degrees, by T_22(t0) ~ 1e3 here.
    s = small_system
    k, m, nocc = 24, 30, 16
    sch = {"fp64": api.sched("fp64"), "fp32": api.sched("fp32"),
           "mixed": api.sched("fp32", low="bf16", n_low=m // 4)}[mode]
    w, _ = chfsi_converge(small_op, s, k, m, sch, passes=15)
    exact = np.linalg.eigvalsh(dense_h(s))[:k]
    # acceptance: eigenvalues within 1e-6 Ha of the FP64 answer (occupied part)
    assert np.abs(w[:nocc] - exact[:nocc]).max() < 1e-6


def test_chfsi_pass_survives_dependent_columns(small_op, small_system):
    """A block with two equal columns stays rank deficient through the
    filter, so plain Cholesky-QR meets a zero pivot.  The pass orthonormalises
    with shifted Cholesky-QR steps instead: the result is orthonormal, keeps
    the other columns' span, and further passes still converge."""
    s = small_system
    k, m = 24, 20
    v0 = np.random.default_rng(4).uniform(0, 1, s.N)
    upper, lower = api.EigenSolver(small_op).computeUpperBoundWithLanczos(None, 20, v0=v0)
    X = np.random.default_rng(5).standard_normal((s.N, k))
    X[:, 7] = X[:, 3]
    Xm = api.Mat(small_op, k, X)
    before = small_op.info()["shifted_orth"]
    sch = api.sched("fp64")
    w = api.chfsi_pass(small_op, Xm, m, 0.0, upper, lower, sch, rotate=True)
    assert small_op.info()["shifted_orth"] > before
    Q = Xm.get()
    assert np.abs(Q.T @ Q - np.eye(k)).max() < 1e-12
    for _ in range(14):
        w = api.chfsi_pass(small_op, Xm, m, w[-1], upper, w[0], sch, rotate=True)
    exact = np.linalg.eigvalsh(dense_h(s))[:k]
    assert np.abs(w[:16] - exact[:16]).max() < 1e-6


def test_fermi_matches_oracle(small_op):
    eig = np.sort(np.random.default_rng(9).uniform(-1, 1, 64))
    kT = 3.166811429e-6 * 500.0
    mu, occ = api.fermi(small_op, eig, 40, kT)
    rmu, rocc = oracle.fermi(eig, 40, kT)
    assert abs(mu - rmu) < 1e-12
    assert np.abs(occ - rocc).max() < 1e-12


def test_density_matches_oracle(small_op, small_system):
    s = small_system
    X, _ = oracle.cholqr(np.random.default_rng(10).standard_normal((s.N, 24)))
    occ = np.linspace(1.0, 0.0, 24)
    rho = api.density(small_op, api.Mat(small_op, 24, X), occ, s.basis)
    ref = oracle.density(X, occ, s.basis)
    # exact-sliced tensor-core mode products on FP32 operands, the states
    # summed in double-FP32
    assert np.linalg.norm(rho - ref) / np.linalg.norm(ref) < 1e-6


def test_density_in_chunks_of_states(small_op, small_system, monkeypatch):
    """A scratch budget of five states' intermediates splits the 24 states
    into five chunks (the last one short), each accumulated into the same
    FP64 density: the result matches the oracle and the one-chunk build."""
    s = small_system
    X, _ = oracle.cholqr(np.random.default_rng(11).standard_normal((s.N, 24)))
    occ = np.linspace(1.0, 0.0, 24)
    Xd = api.Mat(small_op, 24, X)
    whole = api.density(small_op, Xd, occ, s.basis)
    r = [b.r for b in s.basis]
    n = [b.nodal.shape[0] for b in s.basis]
    rp = [(x + 3) // 4 * 4 for x in r]
    per_state = (r[1] * r[2] * rp[0] + r[2] * n[0] * rp[1] + n[1] * n[0] * rp[2]) * 4
    monkeypatch.setenv("TTG_DENSITY_CHUNK_BYTES", str(5 * per_state))
    parts = api.density(small_op, Xd, occ, s.basis)
    ref = oracle.density(X, occ, s.basis)
    assert np.linalg.norm(parts - ref) / np.linalg.norm(ref) < 1e-6
    assert np.linalg.norm(parts - whole) / np.linalg.norm(whole) < 1e-12


def hartree_case(seed=0, r=(12, 10, 8), nq=(40, 36, 30), n=(33, 31, 29), K=7):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((r[2], r[1], r[0]))
    quad, U, grids = [], [], []
    for d in range(3):
        xq = np.sort(rng.uniform(0, 10, nq[d]))
        wq = rng.uniform(0.1, 0.3, nq[d])
        quad.append((xq, wq))
        U.append(rng.standard_normal((nq[d], r[d])))
        grids.append(np.linspace(0, 10, n[d]))
    alpha = np.geomspace(1e-3, 30.0, K)
    omega = rng.uniform(0.1, 1.0, K)
    return alpha, omega, G, quad, U, grids


def test_hartree_matches_oracle():
    """Random core and factors (heavy cancellation: V ~ 100 from O(1) terms).
    Rounding the inputs and intermediates to FP32 alone moves V by 6e-8
    relative here; the tensor-core path measures ~1.3e-7."""
    args = hartree_case()
    V, ms = api.hartree(*args)
    ref = oracle.hartree(*args)
    assert np.linalg.norm(V - ref) / np.linalg.norm(ref) < 3e-7


def write_driver_input(path, s, k, m, passes, X0, a_init=0.0, lanczos=20):
    H, C = s.H, s.C
    with open(path, "wb") as f:
        f.write(struct.pack("<8q", s.N, H.nnz, C.n_rows, C.nnz, k, m, passes, lanczos))
        f.write(struct.pack("<d", a_init))
        for arr, dt in ((H.row_ptr, np.int64), (H.col, np.int32), (H.val, np.float64),
                        (C.row_ptr, np.int64), (C.col, np.int32), (C.val, np.float64),
                        (s.D, np.float64)):
            f.write(np.ascontiguousarray(arr, dt).tobytes())
        f.write(np.asfortranarray(X0).tobytes(order="F"))


def test_cxx_driver_matches_python_api(small_system, tmp_path):
    """The reference-shaped C++ classes (AX, ChebyShevFilter, MultTM,
    EigenSolver) reproduce the oracle's ChFSI loop."""
    from ttdft_public_gb300 import build
    exe = build.build_driver()
    s = small_system
    k, m, passes = 24, 10, 6
    X0 = np.random.default_rng(11).standard_normal((s.N, k))
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    write_driver_input(inp, s, k, m, passes, X0)
    r = subprocess.run([exe, str(inp), str(out), "fp64"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res = np.fromfile(out, dtype=np.float64)
    upper, lower, w = res[0], res[1], res[2:2 + k]
    # oracle loop with the driver's Lanczos bounds (its start vector is its own)
    X = X0.copy()
    a, a0 = 0.0, lower
    for _ in range(passes):
        X = oracle.cheb_filter(s, X, m, a, upper, a0, return_prev=True)
        X, st = oracle.cholqr(X)
        wr, Q, _ = oracle.rayleigh_ritz(s, X, rotate_x=False)
        a0, a = wr[0], wr[-1]
    assert np.abs(w - wr).max() < 1e-9 * np.abs(wr).max()


def test_bad_csr_rejected_before_launch(tiny_system):
    s = tiny_system
    bad_col = s.H.col.copy()
    bad_col[5] = s.N + 3
    H = system.Csr(s.N, s.N, s.H.row_ptr, bad_col, s.H.val)
    with pytest.raises(TtgError) as e:
        api.Operator(api.ProjectHamiltonianSparse(H), 8)
    assert e.value.status == "BAD_CSR"


def test_nonfinite_block_rejected(tiny_op, tiny_system):
    X = np.ones((tiny_system.N, 3))
    X[7, 1] = np.nan
    with pytest.raises(TtgError) as e:
        api.Mat(tiny_op, 3, X)
    assert e.value.status == "NONFINITE"
