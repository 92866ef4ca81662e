"""CPU tests: the oracle against dense numpy/LAPACK restatements (known
answers), and the host operator producer against a dense Kronecker formula."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from ttdft_public_gb300 import system


def dense_h(s):
    H = s.H.to_dense()
    C = s.C.to_dense()
    return H + C.T @ np.diag(s.D) @ C


def test_assembly_matches_dense_kronecker_formula():
    spec = system.small_spec(truncation=0.0)
    s = system.build_system(spec)
    m = s.mats
    kin = 0.5 * (np.kron(np.kron(m["MZ"], m["MY"]), m["DX"]) +
                 np.kron(np.kron(m["MZ"], m["DY"]), m["MX"]) +
                 np.kron(np.kron(m["DZ"], m["MY"]), m["MX"]))
    pot = sum(m["coef"][t] * np.kron(np.kron(m["PZ"][t], m["PY"][t]), m["PX"][t])
              for t in range(len(m["coef"])))
    ref = kin + pot
    got = s.H.to_dense()
    assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()
    # symmetric, and the truncated operator differs only below the threshold
    assert np.abs(ref - ref.T).max() < 1e-12
    s2 = system.build_system(system.small_spec(truncation=1e-6))
    d = s2.H.to_dense()
    kept = d != 0
    assert np.all(np.abs(ref[~kept]) <= 1e-6 + 1e-12)
    assert np.abs(d[kept] - ref[kept]).max() < 1e-12


def test_basis_orthonormal_and_nodal_consistent(tiny_system):
    for b in tiny_system.basis:
        assert np.abs(b.overlap() - np.eye(b.r)).max() < 1e-12
        assert b.nodal[0].max() == 0 and b.nodal[-1].max() == 0


def test_apply_h_matches_dense(tiny_system):
    s = tiny_system
    rng = np.random.default_rng(0)
    X = rng.standard_normal((s.N, 5))
    Y = oracle.apply_h(s, X)
    ref = dense_h(s) @ X
    assert np.abs(Y - ref).max() < 1e-12 * np.abs(ref).max()


def cheb_dense(A, X, m, a, b, a0):
    """Closed form of the scaled recurrence: Y_m = T_m(t(A)) / T_m(t(a0)) X."""
    e, c = (b - a) / 2, (b + a) / 2
    w, V = np.linalg.eigh(A)
    t = (w - c) / e
    t0 = (a0 - c) / e

    def T(mm, x):
        x = np.asarray(x, dtype=float)
        out = np.empty_like(x)
        inside = np.abs(x) <= 1
        out[inside] = np.cos(mm * np.arccos(x[inside]))
        xo = x[~inside]
        out[~inside] = np.sign(xo) ** mm * np.cosh(mm * np.arccosh(np.abs(xo)))
        return out

    p = T(m, t) / T(m, np.array([t0]))[0]
    return V @ (p[:, None] * (V.T @ X))


@pytest.mark.parametrize("return_prev", [False, True])
def test_cheb_filter_matches_closed_form(tiny_system, return_prev):
    s = tiny_system
    A = dense_h(s)
    w = np.linalg.eigvalsh(A)
    k, m = 6, 9
    a, b, a0 = w[k + 2], w[-1] * 1.01, w[0]
    rng = np.random.default_rng(1)
    X = rng.standard_normal((s.N, k))
    got = oracle.cheb_filter(s, X, m, a, b, a0, return_prev=return_prev)
    ref = cheb_dense(A, X, m - 1 if return_prev else m, a, b, a0)
    assert np.abs(got - ref).max() < 1e-10 * np.abs(ref).max()


def test_cheb_filter_degree_one_reference_returns_input(tiny_system):
    s = tiny_system
    X = np.random.default_rng(2).standard_normal((s.N, 3))
    got = oracle.cheb_filter(s, X, 1, 0.5, 5.0, 0.1, return_prev=True)
    assert np.array_equal(got, X)


def test_lanczos_matches_numpy_recurrence(tiny_system):
    s = tiny_system
    A = dense_h(s)
    v0 = np.random.default_rng(3).uniform(0, 1, s.N)
    al, be = oracle.lanczos_T(s, v0, 12)
    v = v0 / np.linalg.norm(v0)
    f = A @ v
    a_ = f @ v
    f = f - a_ * v
    ral, rbe = [a_], []
    vp = np.zeros_like(v)
    for it in range(1, 12):
        b_ = np.linalg.norm(f)
        rbe.append(b_)
        vp, v = v, f / b_
        f = A @ v - b_ * vp
        a_ = v @ f
        f = f - a_ * v
        ral.append(a_)
    rbe.append(np.linalg.norm(f))
    assert np.allclose(al, ral, rtol=1e-10, atol=1e-12)
    assert np.allclose(be, rbe, rtol=1e-10, atol=1e-12)
    up, lo = oracle.lanczos_bounds(s, v0, 12)
    w = np.linalg.eigvalsh(A)
    assert up >= w[-1] - 1e-9 and lo >= w[0] - 1e-9


def test_cholqr_matches_numpy():
    rng = np.random.default_rng(4)
    X = rng.standard_normal((500, 20))
    Q, st = oracle.cholqr(X)
    assert st == 0
    L = np.linalg.cholesky(X.T @ X)
    ref = np.linalg.solve(L, X.T).T
    assert np.abs(Q - ref).max() < 1e-11
    assert np.abs(Q.T @ Q - np.eye(20)).max() < 1e-12
    Xbad = X.copy()
    Xbad[:, 5] = Xbad[:, 3]
    _, st = oracle.cholqr(Xbad)
    assert st != 0


def test_gram_and_rotate():
    rng = np.random.default_rng(5)
    X, Y = rng.standard_normal((300, 7)), rng.standard_normal((300, 7))
    assert np.abs(oracle.gram(X, Y) - X.T @ Y).max() < 1e-12
    Q = rng.standard_normal((7, 7))
    assert np.abs(oracle.rotate(X, Q) - X @ Q).max() < 1e-12


def test_fermi_conserves_electrons():
    eig = np.sort(np.random.default_rng(6).uniform(-1, 1, 40))
    kT = 3.166811429e-6 * 500.0
    mu, occ = oracle.fermi(eig, 24, kT)
    assert abs(2 * occ.sum() - 24) < 1e-7
    assert np.all((occ >= 0) & (occ <= 1))


def test_density_matches_pointwise(tiny_system):
    s = tiny_system
    rng = np.random.default_rng(7)
    X = rng.standard_normal((s.N, 3))
    occ = np.array([1.0, 0.5, 0.25])
    rho = oracle.density(X, occ, s.basis)
    Ux, Uy, Uz = (b.nodal for b in s.basis)
    r = Ux.shape[1]
    for (i, j, l) in [(3, 4, 5), (7, 1, 9), (10, 10, 10)]:
        val = 0.0
        for st in range(3):
            c = X[:, st].reshape(r, r, r)  # (z, y, x)
            psi = np.einsum("zyx,x,y,z->", c, Ux[i], Uy[j], Uz[l])
            val += 2 * occ[st] * psi ** 2
        assert abs(rho[l, j, i] - val) < 1e-12 * max(1.0, abs(val))


def test_hartree_oracle_matches_direct_sum():
    rng = np.random.default_rng(8)
    rx, ry, rz, nq, n = 3, 4, 2, 7, 5
    G = rng.standard_normal((rz, ry, rx))
    quad = [(np.linspace(0, 1, nq), rng.uniform(0.1, 0.2, nq)) for _ in range(3)]
    U = [rng.standard_normal((nq, r)) for r in (rx, ry, rz)]
    grids = [np.linspace(0, 1, n) + 0.01 * d for d in range(3)]
    alpha, omega = np.array([0.5, 3.0]), np.array([1.2, -0.4])
    V = oracle.hartree(alpha, omega, G, quad, U, grids)
    i, j, l = 1, 3, 2
    ref = 0.0
    for t in range(2):
        F = []
        for d, idx in enumerate((i, j, l)):
            xq, wq = quad[d]
            e = wq * np.exp(-alpha[t] * (grids[d][idx] - xq) ** 2)
            F.append(e @ U[d])
        ref += omega[t] * np.einsum("cba,a,b,c->", G, F[0], F[1], F[2])
    assert abs(V[l, j, i] - ref) < 1e-12 * max(1.0, abs(ref))
