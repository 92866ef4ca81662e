"""Synthetic Kohn-Sham systems in a separable (Tucker) basis.

This is the operator producer that feeds the Chebyshev-filtered subspace
iteration.  It restates, for seeded synthetic atoms, what the reference builds
from its input files:

* 1-D Lagrange FEM (quadratic, 3-point Gauss) -- fem/FEM.cc:159-161 (uniform
  nodes), :906-1005 (field/derivative at quadrature points, integration with
  J*w and J^-1*w), Gauss table fem/QuadratureRule.cc:36-47.
* 1-D basis functions with Dirichlet zeros at both ends
  (basis/BasisFunctionReader.h:35-52): orthonormal, exponentially localised
  functions (see make_basis_1d), orthonormal because the Hamiltonian
  assembly assumes it: there is no overlap matrix in Create_Hloc.
* 1-D overlap / stiffness / potential matrices --
  dft/ProjectHamiltonianSparse.cc:577-775.
* H_loc assembly with truncation -- dft/ProjectHamiltonianSparse.cc:330-575
  (done in C++, csrc/gen/assemble_h.cc).
* C_nloc for one separable s-projector per atom --
  dft/ProjectHamiltonianSparse.cc:83-328: C_nloc = D*C with D the coupling,
  C_nloc_trans = C^T, so the nonlocal operator is C^T D C.

Everything here is host-side FP64 (numpy/scipy for the 1-D parts).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import os

import numpy as np
import scipy.linalg

from . import _lib

GAUSS3_X = np.array([-math.sqrt(3.0 / 5.0), 0.0, math.sqrt(3.0 / 5.0)])
GAUSS3_W = np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])


class Fem1D:
    """Uniform 1-D quadratic Lagrange FEM on [x0, x1] with 3-point Gauss.

    Nodes are equispaced (fem/FEM.cc:163-174); quadrature points are ordered
    element by element (fem/FEM.cc:906-944)."""

    def __init__(self, n_el: int, x0: float, x1: float):
        self.n_el = n_el
        self.x0, self.x1 = float(x0), float(x1)
        self.n_nodes = 2 * n_el + 1
        self.nodes = np.linspace(x0, x1, self.n_nodes)
        h = (x1 - x0) / n_el
        self.jac = h / 2.0
        xi = GAUSS3_X
        # shape functions at the reference nodes -1, 0, 1
        self.N = np.stack([xi * (xi - 1) / 2, 1 - xi ** 2, xi * (xi + 1) / 2], axis=1)  # (3q, 3n)
        self.dN = np.stack([xi - 0.5, -2 * xi, xi + 0.5], axis=1)
        left = x0 + h * np.arange(n_el)
        self.xq = (left[:, None] + (xi[None, :] + 1.0) * self.jac).reshape(-1)
        self.wJ = np.tile(GAUSS3_W * self.jac, n_el)            # J * w
        self.wJinv = np.tile(GAUSS3_W / self.jac, n_el)         # J^-1 * w
        self.nq = self.xq.size

    def interp_matrix(self, deriv: bool = False) -> np.ndarray:
        """Dense (nq x n_nodes) matrix taking nodal values to quad values.
        With deriv=True the derivative w.r.t. the reference coordinate (the
        reference integrates it with J^-1*w, fem/FEM.cc:997-1005)."""
        B = np.zeros((self.nq, self.n_nodes))
        S = self.dN if deriv else self.N
        for e in range(self.n_el):
            B[3 * e:3 * e + 3, 2 * e:2 * e + 3] += S
        return B

    def integrate(self, fq: np.ndarray) -> float:
        return float(fq @ self.wJ)


@dataclasses.dataclass
class Basis1D:
    fem: Fem1D
    nodal: np.ndarray      # (n_nodes, r) nodal values incl. the Dirichlet zeros
    quad: np.ndarray       # (nq, r) values at quad points
    dquad: np.ndarray      # (nq, r) reference-coordinate derivative at quad points
    centres: np.ndarray    # (r,)

    @property
    def r(self) -> int:
        return self.nodal.shape[1]

    def overlap(self) -> np.ndarray:
        return self.quad.T @ (self.fem.wJ[:, None] * self.quad)

    def stiffness(self) -> np.ndarray:
        return self.dquad.T @ (self.fem.wJinv[:, None] * self.dquad)

    def weighted(self, g: np.ndarray) -> np.ndarray:
        """int psi_i g psi_j for g given at quad points."""
        return self.quad.T @ ((self.fem.wJ * g)[:, None] * self.quad)

    def project(self, g: np.ndarray) -> np.ndarray:
        """int psi_i g for g given at quad points."""
        return self.quad.T @ (self.fem.wJ * g)


def make_basis_1d(fem: Fem1D, r: int, width: float = 0.6) -> Basis1D:
    """r orthonormal, exponentially localised 1-D basis functions.

    Gaussians on r uniformly spaced centres (spacing s, width `width`*s),
    zero at both Dirichlet ends (basis/BasisFunctionReader.h:35-52), made
    orthonormal with the symmetric (Loewdin) transform S^-1/2, which keeps
    each function centred on its own node and ordered by centre, so H_loc is
    banded in each Tucker index.  The reference instead localises the lowest
    eigenfunctions of a separable Hamiltonian with a per-centre penalty inside
    their span (basis/BasisLocalization.cc:247-306); functions restricted to
    that span decay only algebraically, and at a truncation of 1e-8 the
    resulting H_loc is essentially dense, which is why this basis is used."""
    L = fem.x1 - fem.x0
    s = L / r
    centres = fem.x0 + (np.arange(r) + 0.5) * s
    nodes = fem.nodes[1:-1]
    Phi = np.exp(-(nodes[:, None] - centres[None, :]) ** 2 / (2.0 * (width * s) ** 2))
    B = fem.interp_matrix()[:, 1:-1]
    M = B.T @ (fem.wJ[:, None] * B)
    Sm = Phi.T @ M @ Phi
    w, U = np.linalg.eigh(0.5 * (Sm + Sm.T))
    C = Phi @ (U @ np.diag(w ** -0.5) @ U.T)
    nodal = np.zeros((fem.n_nodes, r))
    nodal[1:-1] = C
    Bf = fem.interp_matrix()
    dBf = fem.interp_matrix(deriv=True)
    return Basis1D(fem, nodal, Bf @ nodal, dBf @ nodal, centres)


def place_atoms(n_atoms: int, box: float, min_sep: float, margin: float, seed: int) -> np.ndarray:
    """Seeded uniform random positions with rejection on minimum separation."""
    rng = np.random.default_rng(seed)
    pos = []
    tries = 0
    while len(pos) < n_atoms:
        p = rng.uniform(margin, box - margin, size=3)
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("could not place atoms with the requested separation")
        if all(np.linalg.norm(p - q) >= min_sep for q in pos):
            pos.append(p)
    return np.array(pos)


@dataclasses.dataclass
class SystemSpec:
    """One synthetic configuration (all lengths in bohr, energies in Ha)."""
    name: str
    n_atoms: int
    box: float
    n_el: int                 # FEM elements per direction
    rank: int                 # Tucker basis rank per direction
    n_states: int
    degree: int
    z_val: float = 3.0        # electrons per atom == Gaussian-well depth
    sigma: float = 0.6        # Gaussian-well width
    min_sep: float = 3.0
    margin: float = 2.5
    nonlocal_width: float = 0.0   # 0: no nonlocal part
    nonlocal_coupling: float = 0.0
    truncation: float = 1e-8
    c_truncation: float = 1e-10
    # Pattern-only envelope (Ha; 0: off): per atom -A exp(-|r-R|^2 / (2 s^2))
    # with s = pattern_envelope_sigma.  The frozen pattern then also keeps the
    # entries that this potential, added to the wells, lifts above the
    # truncation; the stored values stay the wells' operator.
    pattern_envelope: float = 0.0
    pattern_envelope_sigma: float = 1.6
    basis_width: float = 0.6      # Gaussian width / centre spacing of the 1-D basis
    seed: int = 1234

    @property
    def n_electrons(self) -> int:
        return int(round(self.z_val * self.n_atoms))


# The configurations the benchmarks and tests are quoted on.  Sizes follow the
# reference's documented workloads: an 8-atom CPU-sized case, a 64-atom case
# with nonlocal projectors, and a 512-atom case.
CONFIGS = {
    "atoms8": SystemSpec("atoms8", 8, 20.0, 60, 20, 16, 20),
    "atoms64": SystemSpec("atoms64", 64, 32.0, 120, 40, 160, 30,
                          nonlocal_width=1.0, nonlocal_coupling=0.5),
    "atoms512": SystemSpec("atoms512", 512, 64.0, 240, 80, 1200, 40,
                           nonlocal_width=1.0, nonlocal_coupling=0.5),
}


def small_spec(name="tiny", n_atoms=2, box=10.0, n_el=16, rank=6, n_states=8, degree=8,
               with_nonlocal=True, seed=7, truncation=1e-8) -> SystemSpec:
    return SystemSpec(name, n_atoms, box, n_el, rank, n_states, degree,
                      min_sep=2.0, margin=2.0,
                      nonlocal_width=1.0 if with_nonlocal else 0.0,
                      nonlocal_coupling=0.5 if with_nonlocal else 0.0,
                      truncation=truncation, seed=seed)


@dataclasses.dataclass
class Csr:
    n_rows: int
    n_cols: int
    row_ptr: np.ndarray   # int64 (n_rows+1)
    col: np.ndarray       # int32
    val: np.ndarray       # float64

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    def to_dense(self) -> np.ndarray:
        A = np.zeros((self.n_rows, self.n_cols))
        for i in range(self.n_rows):
            s, e = self.row_ptr[i], self.row_ptr[i + 1]
            A[i, self.col[s:e]] = self.val[s:e]
        return A

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.row_ptr), shape=(self.n_rows, self.n_cols))


@dataclasses.dataclass
class KSSystem:
    spec: SystemSpec
    atoms: np.ndarray
    basis: list            # [Basis1D]*3
    H: Csr                 # H_loc (N x N)
    C: Csr                 # C (nproj x N): the projector overlaps
    D: np.ndarray          # (nproj,) couplings; C_nloc = D*C, C_nloc_trans = C^T
    mats: dict             # 1-D matrices used by the assembly

    @property
    def N(self) -> int:
        return self.H.n_rows


def _gauss(x, centre, sigma):
    return np.exp(-(x - centre) ** 2 / (2.0 * sigma ** 2))


def local_potential_factors(spec: SystemSpec, atoms: np.ndarray):
    """V_loc(r) = -sum_a Z exp(-|r-R_a|^2/(2 sigma^2)) as a CP sum of 1-D
    Gaussians: coefficients and per-axis factor callables."""
    coef = -spec.z_val * np.ones(len(atoms))
    return coef


def assemble_hloc(basis, coef, fx, fy, fz, truncation, envelope=None) -> tuple[Csr, dict]:
    """Build the 1-D matrices and call the C++ row-parallel assembly.

    fx, fy, fz: (nterm, nq) CP potential factors at the quad points.
    envelope: None, or (coef, fx, fy, fz) of a second CP potential that widens
    the pattern only (ttg_host_assemble_hloc_pattern)."""
    bx, by, bz = basis
    r = np.array([bx.r, by.r, bz.r], dtype=np.int32)
    MX, MY, MZ = bx.overlap(), by.overlap(), bz.overlap()
    DX, DY, DZ = bx.stiffness(), by.stiffness(), bz.stiffness()
    nterm = len(coef)
    PX = np.ascontiguousarray(np.stack([bx.weighted(fx[t]) for t in range(nterm)])) if nterm else np.zeros((0, bx.r, bx.r))
    PY = np.ascontiguousarray(np.stack([by.weighted(fy[t]) for t in range(nterm)])) if nterm else np.zeros((0, by.r, by.r))
    PZ = np.ascontiguousarray(np.stack([bz.weighted(fz[t]) for t in range(nterm)])) if nterm else np.zeros((0, bz.r, bz.r))
    lib = _lib.host()
    N = int(r.prod())
    row_ptr = np.zeros(N + 1, dtype=np.int64)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (MX, MY, MZ, DX, DY, DZ)]
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    P = [np.ascontiguousarray(a, dtype=np.float64) for a in (PX, PY, PZ)]
    ptr = _lib.ptr
    cp, vp = ctypes.c_void_p(), ctypes.c_void_p()
    if envelope is None:
        rc = lib.ttg_host_assemble_hloc_once(ptr(r), *[ptr(a) for a in args], nterm, ptr(coef),
                                             *[ptr(a) for a in P], ctypes.c_double(truncation),
                                             ctypes.c_double(1e-15), ptr(row_ptr),
                                             ctypes.byref(cp), ctypes.byref(vp))
    else:
        ecoef = np.ascontiguousarray(envelope[0], dtype=np.float64)
        Q = [np.ascontiguousarray(np.stack([b.weighted(f[t]) for t in range(len(ecoef))]),
                                  dtype=np.float64)
             for b, f in zip(basis, envelope[1:])]
        rc = lib.ttg_host_assemble_hloc_pattern(ptr(r), *[ptr(a) for a in args], nterm,
                                                ptr(coef), *[ptr(a) for a in P], len(ecoef),
                                                ptr(ecoef), *[ptr(a) for a in Q],
                                                ctypes.c_double(truncation),
                                                ctypes.c_double(1e-15), ptr(row_ptr),
                                                ctypes.byref(cp), ctypes.byref(vp))
    if rc != 0:
        raise RuntimeError(f"H_loc assembly failed ({rc})")
    nnz = int(row_ptr[-1])
    try:
        col = np.ctypeslib.as_array(ctypes.cast(cp, ctypes.POINTER(ctypes.c_int32)), (max(nnz, 1),))[:nnz].copy()
        val = np.ctypeslib.as_array(ctypes.cast(vp, ctypes.POINTER(ctypes.c_double)), (max(nnz, 1),))[:nnz].copy()
    finally:
        lib.ttg_host_free(cp)
        lib.ttg_host_free(vp)
    mats = dict(MX=MX, MY=MY, MZ=MZ, DX=DX, DY=DY, DZ=DZ, PX=PX, PY=PY, PZ=PZ, coef=coef)
    return Csr(N, N, row_ptr, col, val), mats


def assemble_cnloc(basis, cx, cy, cz, tol) -> Csr:
    r = np.array([b.r for b in basis], dtype=np.int32)
    nproj = cx.shape[0]
    lib = _lib.host()
    ptr = _lib.ptr
    row_ptr = np.zeros(nproj + 1, dtype=np.int64)
    cx, cy, cz = (np.ascontiguousarray(a, dtype=np.float64) for a in (cx, cy, cz))
    rc = lib.ttg_host_assemble_cnloc(ptr(r), nproj, ptr(cx), ptr(cy), ptr(cz),
                                     ctypes.c_double(tol), ptr(row_ptr), None, None)
    if rc != 0:
        raise RuntimeError("C_nloc assembly failed")
    nnz = int(row_ptr[-1])
    col = np.zeros(nnz, dtype=np.int32)
    val = np.zeros(nnz, dtype=np.float64)
    rc = lib.ttg_host_assemble_cnloc(ptr(r), nproj, ptr(cx), ptr(cy), ptr(cz),
                                     ctypes.c_double(tol), ptr(row_ptr), ptr(col), ptr(val))
    if rc != 0:
        raise RuntimeError("C_nloc assembly failed")
    return Csr(nproj, int(r.prod()), row_ptr, col, val)


def build_system(spec: SystemSpec, cache_dir: str | None = None) -> KSSystem:
    """Generate atoms, basis, H_loc and C for a spec (deterministic)."""
    if cache_dir:
        env = f"_env{spec.pattern_envelope:g}_{spec.pattern_envelope_sigma:g}" \
            if spec.pattern_envelope > 0 else ""
        path = os.path.join(cache_dir, f"{spec.name}_{spec.seed}_{spec.truncation:g}{env}.npz")
        if os.path.exists(path):
            return _load(spec, path)
    atoms = place_atoms(spec.n_atoms, spec.box, spec.min_sep, spec.margin, spec.seed)
    fem = Fem1D(spec.n_el, 0.0, spec.box)
    basis = []
    fac = []
    for d in range(3):
        g = np.stack([_gauss(fem.xq, atoms[a, d], spec.sigma) for a in range(spec.n_atoms)])
        fac.append(g)
        basis.append(make_basis_1d(fem, spec.rank, spec.basis_width))
    coef = -spec.z_val * np.ones(spec.n_atoms)
    envelope = None
    if spec.pattern_envelope > 0:
        envelope = (-spec.pattern_envelope * np.ones(spec.n_atoms),
                    *[np.stack([_gauss(fem.xq, atoms[a, d], spec.pattern_envelope_sigma)
                                for a in range(spec.n_atoms)]) for d in range(3)])
    H, mats = assemble_hloc(basis, coef, fac[0], fac[1], fac[2], spec.truncation, envelope)
    if spec.nonlocal_width > 0:
        s = spec.nonlocal_width
        norm = math.pi ** (-0.25) * s ** (-0.5)   # unit-norm 1-D Gaussian
        cs = [np.stack([basis[d].project(norm * _gauss(fem.xq, atoms[a, d], s))
                        for a in range(spec.n_atoms)]) for d in range(3)]
        C = assemble_cnloc(basis, cs[0], cs[1], cs[2], spec.c_truncation)
        D = spec.nonlocal_coupling * np.ones(spec.n_atoms)
    else:
        C = Csr(0, H.n_cols, np.zeros(1, dtype=np.int64), np.zeros(0, np.int32), np.zeros(0))
        D = np.zeros(0)
    sysm = KSSystem(spec, atoms, basis, H, C, D, mats)
    if cache_dir:
        os.makedirs(cache_dir, exist_ok=True)
        _save(sysm, path)
    return sysm


def _save(s: KSSystem, path: str):
    b = s.basis
    np.savez(path, atoms=s.atoms, Hp=s.H.row_ptr, Hc=s.H.col, Hv=s.H.val,
             Cp=s.C.row_ptr, Cc=s.C.col, Cv=s.C.val, Cn=np.array([s.C.n_rows]), D=s.D,
             **{f"nodal{d}": b[d].nodal for d in range(3)},
             **{f"quad{d}": b[d].quad for d in range(3)},
             **{f"dquad{d}": b[d].dquad for d in range(3)},
             **{f"cen{d}": b[d].centres for d in range(3)})


def _load(spec: SystemSpec, path: str) -> KSSystem:
    z = np.load(path)
    fem = Fem1D(spec.n_el, 0.0, spec.box)
    basis = [Basis1D(fem, z[f"nodal{d}"], z[f"quad{d}"], z[f"dquad{d}"], z[f"cen{d}"]) for d in range(3)]
    N = spec.rank ** 3
    H = Csr(N, N, z["Hp"], z["Hc"], z["Hv"])
    C = Csr(int(z["Cn"][0]), N, z["Cp"], z["Cc"], z["Cv"])
    return KSSystem(spec, z["atoms"], basis, H, C, z["D"], {})


def hartree_blob_case(rank=60, n_blobs=64, seed=303, width=1.0, n_el=120, box=32.0):
    """The standalone Hartree workload: a Tucker density with core rank^3 and
    factors at the 3 n_el quadrature points per direction of a box-bohr mesh
    (360 for 120 elements), from n_blobs seeded Gaussian charge blobs (HOSVD
    of their sum, computed from the blobs' separable form), the 35-term kernel
    expansion, output on the quadrature grid.  Returns (alpha, omega, G as
    (rz, ry, rx), quad = [(xq, wq)] * 3, U = [nq x rank] * 3, grids)."""
    from .kernel_expansion import coulomb_expansion
    fem = Fem1D(n_el, 0.0, box)
    xq, wq = fem.xq, fem.wJ
    atoms = place_atoms(n_blobs, box, 3.0, 2.5, seed)
    norm = 1.0 / (math.pi * width * width) ** 1.5
    g = [np.exp(-(xq[None, :] - atoms[:, d][:, None]) ** 2 / width ** 2) for d in range(3)]
    U = []
    for d in range(3):
        o = [e for e in range(3) if e != d]
        # mode-d Gram of sum_a norm gx_a (x) gy_a (x) gz_a
        S = (g[o[0]] @ g[o[0]].T) * (g[o[1]] @ g[o[1]].T) * norm * norm
        w, V = np.linalg.eigh(g[d].T @ S @ g[d])
        U.append(V[:, ::-1][:, :rank].copy())
    P = [U[d].T @ g[d].T for d in range(3)]                  # (rank, n_blobs)
    G = norm * np.einsum("ia,ja,ka->kji", P[0], P[1], P[2])  # (rz, ry, rx), x fastest
    alpha, omega = coulomb_expansion()
    return alpha, omega, G, [(xq, wq)] * 3, U, [xq] * 3
