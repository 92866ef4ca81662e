"""FP64 CPU oracle for the ChFSI hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this package, and only as the checker or the timed CPU
baseline.  The product path (ttdft_public_gb300) never calls it.

The heavy loops are plain C with OpenMP (oracle.c, built by oracle/Makefile);
the dense k x k eigensolves use numpy/scipy LAPACK, which is allowed here
because this is the oracle.  Each function names the reference code it
restates.  Parity to the reference binary is unpinned (it cannot be built
here and ships no golden vectors); the oracle is pinned by known-answer
tests against dense numpy formulas and LAPACK, by committed golden fixtures
under tests/golden/, and by invariants.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np
import scipy.linalg

_DIR = os.path.dirname(os.path.abspath(__file__))
_lib = None

c_i64, c_i32, c_dbl, c_vp = ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p


def build(force: bool = False) -> str:
    path = os.path.join(_DIR, "liboracle.so")
    src = os.path.join(_DIR, "oracle.c")
    if force or not os.path.exists(path) or os.path.getmtime(src) > os.path.getmtime(path):
        r = subprocess.run(["make", "-C", _DIR, "-B", "liboracle.so"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return path


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        csr = [c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]
        L.or_apply_h.argtypes = csr + [c_vp, c_i32, c_vp]
        L.or_cheb_filter.argtypes = csr + [c_vp, c_i32, c_i32, c_dbl, c_dbl, c_dbl, c_i32, c_i32]
        L.or_lanczos.argtypes = csr + [c_vp, c_i32, c_vp, c_vp]
        L.or_gram.argtypes = [c_i64, c_i32, c_vp, c_vp, c_vp]
        L.or_cholqr.argtypes = [c_i64, c_i32, c_vp]
        L.or_cholqr.restype = ctypes.c_int
        L.or_rotate.argtypes = [c_i64, c_i32, c_vp, c_vp]
        L.or_fermi.argtypes = [c_vp, c_i32, c_i32, c_dbl, c_i32, c_vp, c_vp]
        L.or_fermi.restype = ctypes.c_int
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(c_vp)


def _csr_args(sysm):
    H, C, D = sysm.H, sysm.C, sysm.D
    keep = (np.ascontiguousarray(H.row_ptr, np.int64), np.ascontiguousarray(H.col, np.int32),
            np.ascontiguousarray(H.val, np.float64), np.ascontiguousarray(C.row_ptr, np.int64),
            np.ascontiguousarray(C.col, np.int32), np.ascontiguousarray(C.val, np.float64),
            np.ascontiguousarray(D, np.float64))
    args = [H.n_rows, _p(keep[0]), _p(keep[1]), _p(keep[2]), C.n_rows, _p(keep[3]), _p(keep[4]),
            _p(keep[5]), _p(keep[6])]
    return args, keep


def threads() -> int:
    return lib().or_num_threads()


def apply_h(sysm, X: np.ndarray) -> np.ndarray:
    """(H_loc + C^T D C) X -- ChebyShevFilter.cc:97-124."""
    X = np.asfortranarray(X, np.float64)
    Y = np.zeros_like(X, order="F")
    args, keep = _csr_args(sysm)
    lib().or_apply_h(*args, _p(X), X.shape[1], _p(Y))
    return Y


def cheb_filter(sysm, X: np.ndarray, m: int, a: float, b: float, a0: float,
                return_prev: bool = False, steps_limit: int = -1) -> np.ndarray:
    """ChebyShevFilter::computeFilteredSubspace (ChebyShevFilter.cc:34-189)."""
    X = np.array(X, dtype=np.float64, order="F", copy=True)
    args, keep = _csr_args(sysm)
    lib().or_cheb_filter(*args, _p(X), X.shape[1], int(m), float(a), float(b), float(a0),
                         1 if return_prev else 0, int(steps_limit))
    return X


def lanczos_T(sysm, v0: np.ndarray, maxit: int):
    v0 = np.ascontiguousarray(v0, np.float64)
    al = np.zeros(maxit)
    be = np.zeros(maxit)
    args, keep = _csr_args(sysm)
    lib().or_lanczos(*args, _p(v0), maxit, _p(al), _p(be))
    return al, be


def lanczos_bounds(sysm, v0: np.ndarray, maxit: int):
    """EigenSolver::computeUpperBoundWithLanczos (EigenSolver.cc:186-388)."""
    al, be = lanczos_T(sysm, v0, maxit)
    T = np.diag(al) + np.diag(be[:-1], 1) + np.diag(be[:-1], -1)
    w = np.linalg.eigvalsh(T)
    return be[-1] + abs(w[-1]), w[0]


def gram(X, Y) -> np.ndarray:
    """MultTM::mult (MultTm.cu:86-224): X^T Y."""
    X = np.asfortranarray(X, np.float64)
    Y = np.asfortranarray(Y, np.float64)
    k = X.shape[1]
    S = np.zeros((k, k), order="F")
    lib().or_gram(X.shape[0], k, _p(X), _p(Y), _p(S))
    return S


def cholqr(X):
    """MultTM::orth (MultTm.cu:226-467).  Returns (X_orth, status)."""
    X = np.array(X, dtype=np.float64, order="F", copy=True)
    st = lib().or_cholqr(X.shape[0], X.shape[1], _p(X))
    return X, st


def rotate(X, Q):
    X = np.array(X, dtype=np.float64, order="F", copy=True)
    Q = np.asfortranarray(Q, np.float64)
    lib().or_rotate(X.shape[0], X.shape[1], _p(X), _p(Q))
    return X


def normalize_signs(V: np.ndarray) -> np.ndarray:
    """Largest-magnitude component of each column positive (same convention
    as the GPU eigensolver)."""
    V = np.array(V, copy=True)
    idx = np.argmax(np.abs(V), axis=0)
    sg = np.sign(V[idx, np.arange(V.shape[1])])
    sg[sg == 0] = 1
    return V * sg


def eigh(A):
    """Dense symmetric eig, ascending (EigenSolver.cc:30-184: SLEPc EPSLAPACK
    with divide & conquer); LAPACK's dsyevd via scipy."""
    A = 0.5 * (A + A.T)
    w, V = scipy.linalg.eigh(A, driver="evd")
    return w, normalize_signs(V)


def rayleigh_ritz(sysm, X, rotate_x: bool = True):
    """main.cc:1066-1115 (+ rotation main.cc:1186-1207)."""
    HX = apply_h(sysm, X)
    P = gram(X, HX)
    w, Q = eigh(P)
    return w, Q, (rotate(X, Q) if rotate_x else X)


def chfsi_pass(sysm, X, m, a, b, a0, return_prev=False):
    X = cheb_filter(sysm, X, m, a, b, a0, return_prev=return_prev)
    X, st = cholqr(X)
    if st:
        raise RuntimeError("oracle Cholesky failed")
    return rayleigh_ritz(sysm, X)


def fermi(eig, n_electrons: int, kT: float, max_iter: int = 20):
    eig = np.ascontiguousarray(eig, np.float64)
    occ = np.zeros_like(eig)
    mu = ctypes.c_double()
    lib().or_fermi(_p(eig), eig.size, int(n_electrons), float(kT), int(max_iter),
                   ctypes.byref(mu), _p(occ))
    return mu.value, occ


def density(X: np.ndarray, occ: np.ndarray, basis) -> np.ndarray:
    """rho_nodal = sum_i 2 f_i (c_i x1 Ux x2 Uy x3 Uz)^2
    (ProjectHamiltonianSparse.cc:1021-1075); returns (nz, ny, nx)."""
    Ux, Uy, Uz = (b.nodal for b in basis)
    rx, ry, rz = Ux.shape[1], Uy.shape[1], Uz.shape[1]
    rho = np.zeros((Uz.shape[0], Uy.shape[0], Ux.shape[0]))
    for s in range(X.shape[1]):
        c = X[:, s].reshape(rz, ry, rx)
        psi = np.einsum("zyx,ix,jy,lz->lji", c, Ux, Uy, Uz, optimize=True)
        rho += 2.0 * occ[s] * psi * psi
    return rho


def expansion_factor(alpha, x, xq, wq, U):
    """F_t[i, a] = sum_q wq exp(-alpha_t (x_i - xq)^2) U[q, a]  (KSDFTPotential.cc:509-523)."""
    E = np.exp(-alpha[:, None, None] * (x[None, :, None] - xq[None, None, :]) ** 2)
    return np.einsum("tiq,q,qa->tia", E, wq, U, optimize=True)


def expansion_kernel_exact(alpha, x, edges, xq):
    """The factor integrals of KSDFTPotential.cc:509-523 without quadrature
    error: K_t[i, q] such that sum_q K_t[i, q] U[q, a] is
    int exp(-alpha_t (x_i - y)^2) u_a(y) dy exactly, u_a the quadratic through
    U's values at each element's three quadrature points (product
    integration: per element the moments int t^k exp(-alpha t^2) dt, k <= 2,
    in closed form with erf).  expansion_factor's sum, by contrast, samples
    exp(-alpha_t (x_i - y)^2) at the quadrature points, which the narrow terms
    of the expansion (widths down to 5e-3 bohr) do not resolve.
    Returns (t, len(x), len(xq))."""
    import scipy.special
    alpha = np.asarray(alpha, np.float64)
    n_el = edges.size - 1
    mid = 0.5 * (edges[:-1] + edges[1:])
    se = xq.reshape(n_el, 3) - mid[:, None]          # quadrature points about the element centre
    # coefficients of the quadratic in s = y - mid_e through the three points
    Vinv = np.linalg.inv(np.stack([np.ones_like(se), se, se ** 2], axis=2))   # (e, k, q)
    ta = edges[None, :-1] - x[:, None]                                          # (i, e): t = y - x_i
    tb = edges[None, 1:] - x[:, None]
    xi = x[:, None] - mid[None, :]                                              # s = t + xi
    K = np.zeros((alpha.size, x.size, xq.size))
    for t, al in enumerate(alpha):
        ea, eb = np.exp(-al * ta * ta), np.exp(-al * tb * tb)
        sa = math.sqrt(al)
        I0 = 0.5 * math.sqrt(math.pi / al) * (scipy.special.erf(sa * tb)
                                              - scipy.special.erf(sa * ta))
        I1 = -(eb - ea) / (2.0 * al)
        I2 = I0 / (2.0 * al) - (tb * eb - ta * ea) / (2.0 * al)
        # moments of s^k over the element, s = t + (x_i - mid_e)
        M0 = I0
        M1 = xi * I0 + I1
        M2 = xi * xi * I0 + 2.0 * xi * I1 + I2
        Kt = (np.einsum("ie,eq->ieq", M0, Vinv[:, 0, :]) + np.einsum("ie,eq->ieq", M1, Vinv[:, 1, :])
              + np.einsum("ie,eq->ieq", M2, Vinv[:, 2, :]))
        K[t] = Kt.reshape(x.size, xq.size)
    return K


def hartree(alpha, omega, G, quad, Uq, grids, kernels=None):
    """V = sum_t omega_t G x1 Fx_t x2 Fy_t x3 Fz_t (KSDFTPotential.cc:269-340, 601-658).
    G as (rz, ry, rx); returns (nz, ny, nx).  kernels: optional per-direction
    K_t (expansion_kernel_exact) in place of the quadrature sums."""
    alpha = np.asarray(alpha, np.float64)
    if kernels is None:
        F = [expansion_factor(alpha, grids[d], quad[d][0], quad[d][1], Uq[d]) for d in range(3)]
    else:
        F = [np.einsum("tiq,qa->tia", kernels[d], Uq[d], optimize=True) for d in range(3)]
    V = np.zeros((grids[2].size, grids[1].size, grids[0].size))
    for t in range(alpha.size):
        V += omega[t] * np.einsum("cba,ia,jb,lc->lji", G, F[0][t], F[1][t], F[2][t], optimize=True)
    return V


def hartree_energy(alpha, omega, G, quad, Uq):
    """1/2 sum_qq' w rho K w rho of a Tucker density on its quadrature grid as
    1/2 sum_t omega_t <G, G x1 Kx_t x2 Ky_t x3 Kz_t>, Kd_t = (W U)^T E_t (W U)
    (the Hartree term of main.cc:1315-1401).  G as (rz, ry, rx)."""
    alpha = np.asarray(alpha, np.float64)
    Kd = []
    for d in range(3):
        x, w = quad[d]
        E = np.exp(-alpha[:, None, None] * (x[None, :, None] - x[None, None, :]) ** 2)
        WU = w[:, None] * Uq[d]
        Kd.append(np.einsum("qa,tqp,pb->tab", WU, E, WU, optimize=True))
    e = 0.0
    for t in range(alpha.size):
        T = np.einsum("cba,ia,jb,lc->lji", G, Kd[0][t], Kd[1][t], Kd[2][t], optimize=True)
        e += omega[t] * float(np.sum(G * T))
    return 0.5 * e


def sad_density(atoms, grids, z_val=3.0, width=1.0):
    """Superposition of atomic densities (InitialGuess.cc:573-681): each atom a
    normalised Gaussian of z_val electrons (the synthetic atoms' radial
    density), evaluated on the tensor grid; returns (nz, ny, nx)."""
    x, y, z = grids
    rho = np.zeros((z.size, y.size, x.size))
    norm = z_val / (np.pi * width ** 2) ** 1.5
    for R in atoms:
        gx = np.exp(-(x - R[0]) ** 2 / width ** 2)
        gy = np.exp(-(y - R[1]) ** 2 / width ** 2)
        gz = np.exp(-(z - R[2]) ** 2 / width ** 2)
        rho += norm * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return rho
