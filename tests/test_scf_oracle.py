"""CPU tests of the SCF oracle pieces (known answers / invariants)."""
import math

import numpy as np

from oracle import scf as oscf
from ttdft_public_gb300 import scf
from ttdft_public_gb300.kernel_expansion import coulomb_expansion, expansion_error


def test_coulomb_expansion_accuracy():
    a, w = coulomb_expansion()
    assert len(a) == 35
    assert expansion_error(a, w) < 2e-5
    assert np.all(w > 0)          # no cancellation in the FP32 contraction


def test_sthosvd_error_bound_and_exact_low_rank():
    rng = np.random.default_rng(0)
    # exact rank (3, 2, 4) tensor is recovered to rounding
    core = rng.standard_normal((3, 2, 4))
    U = [np.linalg.qr(rng.standard_normal((n, r)))[0] for n, r in ((9, 3), (7, 2), (8, 4))]
    T = oscf.reconstruct(core, U)
    c2, U2 = oscf.sthosvd(T, 1e-6, 64)
    assert c2.shape == (3, 2, 4)
    assert np.abs(oscf.reconstruct(c2, U2) - T).max() < 1e-10 * np.abs(T).max()
    # a generic tensor: relative Frobenius error <= eps
    T = rng.standard_normal((6, 7, 8)) + np.einsum("i,j,k->kji", *[np.arange(n) for n in (8, 7, 6)])
    eps = 1e-2
    c3, U3 = oscf.sthosvd(T, eps, 64)
    err = np.linalg.norm(oscf.reconstruct(c3, U3) - T) / np.linalg.norm(T)
    assert err <= eps * (1 + 1e-9)


def test_lda_exchange_and_low_density_branch():
    rho = np.array([1e-4, 1e-3, 1e-2])         # rs >= 1
    v, e = oscf.lda(rho)
    exch_c = -(3.0 / 4.0) * np.cbrt(3.0 / math.pi)
    g, b1, b2 = -0.1423, 1.0529, 0.3334
    rs = np.cbrt(3.0 / (4 * math.pi * rho))
    ec = g / (1 + b1 * np.sqrt(rs) + b2 * rs)
    assert np.allclose(e, exch_c * rho ** (4 / 3) + ec * rho, rtol=1e-8)
    # in this branch the potential is d(e)/d(rho)
    h = 1e-8 * rho
    de = (oscf.lda(rho + h)[1] - oscf.lda(rho - h)[1]) / (2 * h)
    assert np.allclose(v, de, rtol=1e-5)


def test_small_linear_solve():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((4, 4)) + 4 * np.eye(4)
    b = rng.standard_normal(4)
    assert np.allclose(scf.solve_small(A, b), np.linalg.solve(A, b), rtol=1e-12)


def test_repulsive_energy():
    atoms = np.array([[0.0, 0, 0], [3.0, 0, 0], [0, 4.0, 0]])
    e = scf.repulsive_energy(atoms, 3.0)
    assert abs(e - 9.0 * (1 / 3 + 1 / 4 + 1 / 5)) < 1e-14


def test_hartree_energy_identity():
    """1/2 sum w rho V_H(rho) on the quadrature grid equals the Tucker form
    1/2 sum_t omega_t <G, G x Kx_t x Ky_t x Kz_t> used for the energy."""
    import oracle
    rng = np.random.default_rng(5)
    a, w = coulomb_expansion()
    n, r = (11, 9, 10), (3, 4, 2)
    quad = [(np.sort(rng.uniform(-4, 4, n[d])), rng.uniform(0.2, 1.0, n[d])) for d in range(3)]
    U = [rng.standard_normal((n[d], r[d])) for d in range(3)]
    G = rng.standard_normal((r[2], r[1], r[0]))
    V = oracle.hartree(a, w, G, quad, U, [q[0] for q in quad])
    rho = oscf.reconstruct(np.transpose(G, (2, 1, 0)), U)          # (nz, ny, nx)
    W = np.einsum("l,j,i->lji", quad[2][1], quad[1][1], quad[0][1])
    ref = 0.5 * float(np.sum(W * rho * V))
    e = oracle.hartree_energy(a, w, G, quad, U)
    assert abs(e - ref) < 1e-12 * abs(ref)


def test_oracle_hamiltonian_values(tiny_system):
    """H values of the oracle (pair tables, chunked) against the direct sum
    H_e = kin_e + sum_abc core[a,b,c] P0[a,xi,xj] P1[b,yi,yj] P2[c,zi,zj]."""
    c = oscf.OracleScf(tiny_system, scf.ScfConfig())
    veff = c.veff_from(c.initial_density())
    H = c.hamiltonian(veff)
    core, U = oscf.sthosvd(veff, c.cfg.veff_eps, c.cfg.veff_rank_cap)
    P = [scf.potential_matrices(tiny_system.basis[d], U[d]) for d in range(3)]
    (xi, yi, zi), (xj, yj, zj) = c.I3, c.J3
    ref = c.kin + np.einsum("abc,ae,be,ce->e", core, P[0][:, xi, xj], P[1][:, yi, yj],
                            P[2][:, zi, zj], optimize=True)
    assert np.abs(H.val - ref).max() < 1e-12 * np.abs(ref).max()


def test_anderson_system_from_gram_matches_direct_differences():
    """The mixing system built from the residuals' Gram matrix (as the GPU
    driver keeps it across iterations) equals the one built from the
    differences D_m = F_n - F_m directly (as the oracle does)."""
    from ttdft_public_gb300.scf import anderson_system
    rng = np.random.default_rng(11)
    h, npts = 7, 500
    w = rng.uniform(0.5, 2.0, npts)
    F = [rng.standard_normal(npts) * (1.0 + 0.1 * i) for i in range(h)]
    dot = lambda a, b: float(np.sum(a * b * w))
    G = np.array([[dot(F[i], F[j]) for j in range(h)] for i in range(h)])
    A, b = anderson_system(G)
    D = [F[h - 1] - F[h - 2 - m] for m in range(h - 1)]
    A_ref = np.array([[dot(D[i], D[j]) for j in range(h - 1)] for i in range(h - 1)])
    b_ref = np.array([dot(D[i], F[h - 1]) for i in range(h - 1)])
    scale = np.abs(G).max()
    assert np.abs(A - A_ref).max() < 1e-12 * scale
    assert np.abs(b - b_ref).max() < 1e-12 * scale
