"""Poisson/FEM Hartree fallback -- TEST INFRASTRUCTURE ONLY (the oracle).

Restates the reference's fallback Hartree solve, used when the kernel
expansion is switched off after the first SCF iteration (main.cc:880-907):
PoissonHartreePotentialSolver::solve (hartree/PoissonHartreePotentialSolver.cc:336-385)
and HartreeCalculator's solve and projection onto the quadrature points
(hartree/HartreeCalculator.cc:101-172).

- The Kohn-Sham mesh is extended in every direction by n_outer elements,
  half on each side, whose sizes grow geometrically by `coarsening` out to
  the outer domain; the inner nodes are kept (FEM.cc:799-860).
- Dirichlet values on the outer boundary are sum_n Z_n / |r - R_n|
  (PhiZoverRBoundaryValuesContainer.cc:36-59).
- -Laplace(phi) = 4 pi rho in the weak form: the stiffness operator is the
  Kronecker sum K_x M_y M_z + M_x K_y M_z + M_x M_y K_z of the 1-D matrices of
  the extended mesh, and rho, known at the Kohn-Sham quadrature points and
  zero outside the Kohn-Sham domain, enters as 4 pi int rho N_i.  The
  reference assembles this system in hartree/LinearSolver/, whose sources
  are not in its repository; the weak form here is the standard one.
- The interior unknowns are solved by preconditioned CG (the reference asks
  PETSc for BiCGStab with block Jacobi; the operator is symmetric positive
  definite, so CG reaches the same solution), starting from a given guess
  (the reference starts from the kernel-expansion potential on the first
  call, PoissonHartreePotentialSolver.cc:150-334, 342-362).
- The nodal potential is interpolated to the Kohn-Sham quadrature points.

Quadratic elements and 3-point Gauss rules, as the rest of this build's FEM
(system.Fem1D); fields are (z, y, x) arrays, x fastest.
"""
from __future__ import annotations

import math

import numpy as np

from ttdft_public_gb300.system import GAUSS3_W, GAUSS3_X

_XI = GAUSS3_X
_N = np.stack([_XI * (_XI - 1) / 2, 1 - _XI ** 2, _XI * (_XI + 1) / 2], axis=1)   # (3q, 3n)
_DN = np.stack([_XI - 0.5, -2 * _XI, _XI + 0.5], axis=1)


def extended_edges(x0: float, x1: float, n_el: int, n_outer: int, coarsening: float,
                   outer0: float, outer1: float) -> np.ndarray:
    """Element boundaries of the extended mesh (FEM.cc:799-860): the n_el
    uniform elements of [x0, x1], then n_outer / 2 elements on each side
    whose sizes grow by `coarsening`, the first of size
    s0 = spacing / sum_{i < n_outer/2} coarsening^i with spacing the width
    added on each side."""
    if n_outer % 2 != 0:
        raise ValueError("n_outer must be even")
    inner = np.linspace(x0, x1, n_el + 1)
    half = n_outer // 2
    spacing = ((outer1 - outer0) - (x1 - x0)) / 2.0
    if half == 0 or spacing <= 0:
        return inner
    sizes = spacing / sum(coarsening ** i for i in range(half)) * coarsening ** np.arange(half)
    right = x1 + np.cumsum(sizes)
    left = x0 - np.cumsum(sizes)
    return np.concatenate([left[::-1], inner, right])


class Mesh1D:
    """Quadratic Lagrange elements on given boundaries, 3-point Gauss."""

    def __init__(self, edges: np.ndarray):
        self.edges = np.asarray(edges, np.float64)
        self.n_el = self.edges.size - 1
        self.n_nodes = 2 * self.n_el + 1
        h = np.diff(self.edges)
        self.jac = h / 2.0
        self.nodes = np.empty(self.n_nodes)
        self.nodes[0::2] = self.edges
        self.nodes[1::2] = 0.5 * (self.edges[:-1] + self.edges[1:])
        self.xq = (self.edges[:-1, None] + (_XI[None, :] + 1.0) * self.jac[:, None]).reshape(-1)
        self.wJ = (GAUSS3_W[None, :] * self.jac[:, None]).reshape(-1)
        self.wJinv = (GAUSS3_W[None, :] / self.jac[:, None]).reshape(-1)

    def interp(self, deriv: bool = False) -> np.ndarray:
        """(nq, n_nodes): nodal values to quadrature values (or reference-
        coordinate derivatives)."""
        B = np.zeros((self.xq.size, self.n_nodes))
        S = _DN if deriv else _N
        for e in range(self.n_el):
            B[3 * e:3 * e + 3, 2 * e:2 * e + 3] += S
        return B

    def mass(self) -> np.ndarray:
        B = self.interp()
        return B.T @ (self.wJ[:, None] * B)

    def stiffness(self) -> np.ndarray:
        D = self.interp(deriv=True)
        return D.T @ (self.wJinv[:, None] * D)


def _kron3(A, B, C, u):
    """(A_z (x) B_y (x) C_x) u for u as (z, y, x)."""
    return np.einsum("kc,jb,ia,cba->kji", A, B, C, u, optimize=True)


def solve_hartree(rho_q, inner_edges, nuclei, n_outer=8, coarsening=1.5, outer=None,
                  guess=None, tol=1e-10, max_iter=5000):
    """Hartree potential at the Kohn-Sham quadrature points by the Poisson
    fallback.

    rho_q       : (nz, ny, nx) density at the KS quadrature points
    inner_edges : three arrays of KS element boundaries (x, y, z)
    nuclei      : (n, 4) rows (Z, x, y, z) for the boundary values
    outer       : three (start, end) outer domains (default: 4x the KS box
                  width on each side)
    guess       : optional nodal potential on the extended mesh (z, y, x)
    Returns (phi_q, info) with info = {iterations, residual, meshes, phi_nodes}.
    """
    meshes, inner_off = [], []
    for d in range(3):
        e = np.asarray(inner_edges[d], np.float64)
        x0, x1 = e[0], e[-1]
        o = outer[d] if outer is not None else (x0 - 4 * (x1 - x0), x1 + 4 * (x1 - x0))
        ext = extended_edges(x0, x1, e.size - 1, n_outer, coarsening, o[0], o[1])
        if not np.allclose(ext[n_outer // 2:n_outer // 2 + e.size], e):
            raise ValueError("extended mesh must contain the KS elements")
        meshes.append(Mesh1D(ext))
        inner_off.append(n_outer // 2)
    M = [m.mass() for m in meshes]
    K = [m.stiffness() for m in meshes]
    # 4 pi int rho N_i: KS quadrature points are those of the inner elements
    P = []
    for d in range(3):
        m = meshes[d]
        B = m.interp()
        q0 = 3 * inner_off[d]
        nq = rho_q.shape[2 - d]
        P.append((B[q0:q0 + nq] * m.wJ[q0:q0 + nq, None]).T)          # (n_nodes, nq)
    f = 4.0 * math.pi * _kron3(P[2], P[1], P[0], rho_q)

    nodes = [m.nodes for m in meshes]
    shape = (nodes[2].size, nodes[1].size, nodes[0].size)
    interior = np.zeros(shape, bool)
    interior[1:-1, 1:-1, 1:-1] = True
    # boundary values sum_n Z_n / r on every boundary node
    Zg, Yg, Xg = np.meshgrid(nodes[2], nodes[1], nodes[0], indexing="ij")
    phi_b = np.zeros(shape)
    on_b = ~interior
    for Z, x, y, z in np.asarray(nuclei, np.float64):
        phi_b[on_b] += Z / np.sqrt((Xg[on_b] - x) ** 2 + (Yg[on_b] - y) ** 2
                                   + (Zg[on_b] - z) ** 2)

    def A(u):
        return (_kron3(M[2], M[1], K[0], u) + _kron3(M[2], K[1], M[0], u)
                + _kron3(K[2], M[1], M[0], u))

    diag = (np.einsum("k,j,i->kji", np.diag(M[2]), np.diag(M[1]), np.diag(K[0]))
            + np.einsum("k,j,i->kji", np.diag(M[2]), np.diag(K[1]), np.diag(M[0]))
            + np.einsum("k,j,i->kji", np.diag(K[2]), np.diag(M[1]), np.diag(M[0])))
    b = np.where(interior, f - A(phi_b), 0.0)
    u = np.where(interior, guess, 0.0) if guess is not None else np.zeros(shape)
    r = np.where(interior, b - A(u), 0.0)
    z = np.where(interior, r / diag, 0.0)
    p = z.copy()
    rz = float(np.sum(r * z))
    bnorm = float(np.linalg.norm(b)) or 1.0
    it = 0
    res = float(np.linalg.norm(r)) / bnorm
    while res > tol and it < max_iter:
        Ap = np.where(interior, A(p), 0.0)
        alpha = rz / float(np.sum(p * Ap))
        u += alpha * p
        r -= alpha * Ap
        z = np.where(interior, r / diag, 0.0)
        rz_new = float(np.sum(r * z))
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
        res = float(np.linalg.norm(r)) / bnorm
    phi = u + phi_b
    Bq = []
    for d in range(3):
        m = meshes[d]
        q0 = 3 * inner_off[d]
        nq = rho_q.shape[2 - d]
        Bq.append(m.interp()[q0:q0 + nq])                               # (nq, n_nodes)
    phi_q = _kron3(Bq[2], Bq[1], Bq[0], phi)
    return phi_q, {"iterations": it, "residual": res, "meshes": meshes, "phi_nodes": phi}
