"""Python mirror of the reference's eigensolver interfaces, over libttg's C ABI.

Same class and method names, argument order and meaning as the reference's
C++ classes (the C++ versions live in include/ttdft/*.h):

  ChebyShevFilter.computeFilteredSubspace   eigensolver/ChebyShevFilter.h:31-39
  AX(num_bg, num_wfns), setup_system, perform_ax, free_mata_on_device
                                            eigensolver/Mult.h:30-61
  MultTM.mult / MultTM.orth                 eigensolver/MultTm.h:33-53
  EigenSolver.computeEigenPairsSeq / computeUpperBoundWithLanczos
                                            eigensolver/EigenSolver.h:30-45
  ProjectHamiltonianSparse (operator holder: H_loc, C_nloc, C_nloc_trans)
                                            dft/ProjectHamiltonianSparse.h:97

A `Mat` here is a device-resident dense N x k block (the reference's PETSc
MATDENSE, column-major on the host side).  Errors raise TtgError carrying the
library status instead of terminating the process.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _lib
from ._lib import TtgSched, check, ptr
from .system import Csr

PREC = {"fp64": 0, "fp32": 1, "bf16": 2, "df64": 3}


def sched(high="fp32", low=None, n_low=0, return_prev=False) -> TtgSched:
    """Precision schedule of one filter call: the first n_low degrees in `low`,
    the rest in `high`.  return_prev=True reproduces the reference's return of
    the degree m-1 iterate (eigensolver/ChebyShevFilter.cc:163-176)."""
    low = high if low is None else low
    return TtgSched(PREC[low], PREC[high], int(n_low), 1 if return_prev else 0)


class ProjectHamiltonianSparse:
    """Operator holder: H_loc (N x N), C (nproj x N) and D (nproj).

    The reference stores C_nloc = diag(D) C and C_nloc_trans = C^T
    (dft/ProjectHamiltonianSparse.cc:316-325); both are views of (C, D) here."""

    def __init__(self, H_loc: Csr, C: Csr | None = None, D: np.ndarray | None = None,
                 ranks: tuple | None = None):
        self.H_loc = H_loc
        self.ranks = ranks          # Tucker ranks (rx, ry, rz) of the basis, if known
        if C is None:
            C = Csr(0, H_loc.n_cols, np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0))
            D = np.zeros(0)
        self.C = C
        self.D = np.ascontiguousarray(D, dtype=np.float64)

    @property
    def C_nloc(self):
        return self.C.to_scipy().multiply(self.D[:, None]).tocsr()

    @property
    def C_nloc_trans(self):
        return self.C.to_scipy().T.tocsr()

    @classmethod
    def from_system(cls, s) -> "ProjectHamiltonianSparse":
        return cls(s.H, s.C, s.D, tuple(b.r for b in s.basis))


class Operator:
    """Device-resident operator (ttg_op): H_loc + C^T D C in the row-group
    format, FP64/FP32/BF16 value copies, and the workspace of one stream."""

    def __init__(self, H: ProjectHamiltonianSparse, max_k: int):
        lib = _lib.ttg()
        h, c = H.H_loc, H.C
        self._keep = [np.ascontiguousarray(a) for a in (h.row_ptr, h.col, h.val, c.row_ptr,
                                                         c.col, c.val, H.D)]
        hp, hc, hv, cp, cc, cv, d = self._keep
        hp = hp.astype(np.int64, copy=False)
        cp = cp.astype(np.int64, copy=False)
        handle = ctypes.c_void_p()
        ranks = None if H.ranks is None else np.array(H.ranks, dtype=np.int32)
        check(lib.ttg_op_create_tucker(h.n_rows, ptr(hp), ptr(hc.astype(np.int32, copy=False)),
                                       ptr(hv.astype(np.float64, copy=False)), c.n_rows, ptr(cp),
                                       ptr(cc.astype(np.int32, copy=False)),
                                       ptr(cv.astype(np.float64, copy=False)), ptr(d), ptr(ranks),
                                       int(max_k), ctypes.byref(handle)), "ttg_op_create_tucker")
        self.h = handle
        self.n = h.n_rows
        self.max_k = max_k
        self._keep = None
        self._blocks = weakref.WeakSet()

    def set_rr_precision(self, prec: str):
        """Arithmetic of H X in Rayleigh-Ritz: "df64" (default) or "fp64"."""
        check(_lib.ttg().ttg_op_set_rr_precision(self.h, PREC[prec]), "ttg_op_set_rr_precision")

    def info(self) -> dict:
        inf = _lib.TtgOpInfo()
        check(_lib.ttg().ttg_op_info(self.h, ctypes.byref(inf)), "ttg_op_info")
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def sync(self):
        check(_lib.ttg().ttg_op_sync(self.h), "ttg_op_sync")

    def record(self, slot: int):
        check(_lib.ttg().ttg_op_record(self.h, slot), "ttg_op_record")

    def elapsed_ms(self, s0: int, s1: int) -> float:
        ms = ctypes.c_float()
        check(_lib.ttg().ttg_op_elapsed_ms(self.h, s0, s1, ctypes.byref(ms)), "ttg_op_elapsed_ms")
        return ms.value

    # kinds of ttg_op_kernel_time (include/ttg.h TTG_KT_*)
    KERNEL_KINDS = {"umma_fp32": 0, "tc_fp32": 1, "tc_bf16": 2, "rowgroup": 3, "umma_bf16": 4,
                    "hartree": 5, "density": 6, "orth_gram": 7, "orth_chol": 8,
                    "orth_update": 9, "rr_hx": 10, "rr_gram": 11, "rr_eig": 12, "rr_rotate": 13}

    def kernel_timing(self, enable: bool):
        """Bracket every fused filter-degree launch with CUDA events on the
        operator's stream (off: stop and clear the totals)."""
        check(_lib.ttg().ttg_op_kernel_timing(self.h, 1 if enable else 0), "ttg_op_kernel_timing")

    def kernel_time(self, kind: str):
        """(total device milliseconds, launches) of one kernel kind since
        timing was switched on."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(_lib.ttg().ttg_op_kernel_time(self.h, self.KERNEL_KINDS[kind], ctypes.byref(ms),
                                            ctypes.byref(n)), "ttg_op_kernel_time")
        return ms.value, n.value

    def stream(self) -> int:
        return _lib.ttg().ttg_op_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            for b in list(self._blocks):
                b.close()
            _lib.ttg().ttg_op_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mat:
    """Device-resident N x k FP64 block (the reference's dense Mat)."""

    def __init__(self, op: Operator, k: int, data: np.ndarray | None = None):
        self.op = op
        self.k = k
        handle = ctypes.c_void_p()
        check(_lib.ttg().ttg_block_create(op.h, k, ctypes.byref(handle)), "ttg_block_create")
        self.h = handle
        op._blocks.add(self)
        if data is not None:
            self.set(data)

    def set(self, X: np.ndarray):
        X = np.asfortranarray(X, dtype=np.float64)
        if X.shape != (self.op.n, self.k):
            raise ValueError(f"expected {(self.op.n, self.k)}, got {X.shape}")
        check(_lib.ttg().ttg_block_set(self.h, ptr(X), self.op.n), "ttg_block_set")

    def get(self) -> np.ndarray:
        X = np.zeros((self.op.n, self.k), order="F")
        check(_lib.ttg().ttg_block_get(self.h, ptr(X), self.op.n), "ttg_block_get")
        return X

    def close(self):
        if getattr(self, "h", None):
            _lib.ttg().ttg_block_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AX:
    """eigensolver/Mult.h:30-61.  setup_system uploads the operator once;
    perform_ax writes (H_loc + C^T D C) X into the caller's pre-allocated AX
    (the reference drops this result, eigensolver/MultCuda.cu:781-820)."""

    def __init__(self, num_bg: int, num_wfns: int):
        if num_bg != 1:
            raise ValueError("one GPU: a single band group")
        self.num_wfns = num_wfns
        self.op: Operator | None = None

    def setup_system(self, A: ProjectHamiltonianSparse):
        self.free_mata_on_device()
        self.op = Operator(A, self.num_wfns)

    def perform_ax(self, X: Mat, AXm: Mat):
        check(_lib.ttg().ttg_apply_h(self.op.h, X.h, AXm.h), "ttg_apply_h")

    def free_mata_on_device(self):
        if self.op is not None:
            self.op.close()
            self.op = None


class ChebyShevFilter:
    """eigensolver/ChebyShevFilter.h:29-40.  In place on X.  `precision` selects
    the schedule (default: the reference's arithmetic, FP64, returning the
    degree m-1 iterate as the reference does)."""

    def __init__(self, precision: TtgSched | None = None):
        self.precision = precision if precision is not None else sched("fp64", return_prev=True)

    def computeFilteredSubspace(self, H: ProjectHamiltonianSparse, ax: AX, X: Mat, basisSize: int,
                                m: int, a: float, b: float, a0: float, num_X_blocks: int = 1):
        if basisSize != ax.op.n:
            raise ValueError("basisSize does not match the operator")
        check(_lib.ttg().ttg_cheb_filter(ax.op.h, X.h, int(m), float(a), float(b), float(a0),
                                         self.precision), "ttg_cheb_filter")


class MultTM:
    """eigensolver/MultTm.h:33-53."""

    def mult(self, X: Mat, Y: Mat) -> np.ndarray:
        k = X.k
        S = np.zeros((k, k), order="F")
        check(_lib.ttg().ttg_gram(X.op.h, X.h, Y.h, ptr(S)), "ttg_gram")
        return S

    def orth(self, X: Mat):
        check(_lib.ttg().ttg_chol_qr(X.op.h, X.h), "ttg_chol_qr")


class EigenSolver:
    """eigensolver/EigenSolver.h:30-45."""

    def __init__(self, op: Operator | None = None):
        self.op = op

    def computeEigenPairsSeq(self, A: np.ndarray, numberEigenPairs: int, numGlobalRows: int,
                             eigVals: np.ndarray, eigMat: np.ndarray, lapack: bool = True):
        k = numberEigenPairs
        A = np.asfortranarray(A, dtype=np.float64)
        w = np.zeros(k)
        V = np.zeros((k, k), order="F")
        check(_lib.ttg().ttg_syev(self.op.h, k, ptr(A), ptr(w), ptr(V)), "ttg_syev")
        eigVals[:k] = w
        eigMat[:, :] = V

    def computeUpperBoundWithLanczos(self, H: ProjectHamiltonianSparse, maxLanczosIteration: int,
                                     v0: np.ndarray | None = None, seed: int = 0):
        n = self.op.n
        if v0 is None:
            v0 = np.random.default_rng(seed).uniform(0.0, 1.0, n)
        v0 = np.ascontiguousarray(v0, dtype=np.float64)
        up, lo = ctypes.c_double(), ctypes.c_double()
        check(_lib.ttg().ttg_lanczos_bounds(self.op.h, ptr(v0), int(maxLanczosIteration),
                                            ctypes.byref(up), ctypes.byref(lo)),
              "ttg_lanczos_bounds")
        return up.value, lo.value


def rayleigh_ritz(op: Operator, X: Mat, rotate: bool = True):
    w = np.zeros(X.k)
    check(_lib.ttg().ttg_rayleigh_ritz(op.h, X.h, 1 if rotate else 0, ptr(w), None),
          "ttg_rayleigh_ritz")
    return w


def chfsi_pass(op: Operator, X: Mat, m: int, a: float, b: float, a0: float, sch: TtgSched,
               rotate: bool = True):
    w = np.zeros(X.k)
    check(_lib.ttg().ttg_chfsi_pass(op.h, X.h, int(m), float(a), float(b), float(a0), sch,
                                    1 if rotate else 0, ptr(w)), "ttg_chfsi_pass")
    return w


def fermi(op: Operator, eig: np.ndarray, n_electrons: float, kT: float, max_iter: int = 20):
    eig = np.ascontiguousarray(eig, dtype=np.float64)
    occ = np.zeros_like(eig)
    mu = ctypes.c_double()
    check(_lib.ttg().ttg_fermi(op.h, eig.size, ptr(eig), float(n_electrons), float(kT), max_iter,
                               ctypes.byref(mu), ptr(occ)), "ttg_fermi")
    return mu.value, occ


def density(op: Operator, X: Mat, occ: np.ndarray, basis) -> np.ndarray:
    """Nodal density sum_i 2 f_i psi_i^2 (x fastest), basis = [Basis1D]*3."""
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    U = [np.asfortranarray(b.nodal, dtype=np.float64) for b in basis]
    n = [u.shape[0] for u in U]
    r = [u.shape[1] for u in U]
    rho = np.zeros(n[0] * n[1] * n[2])
    check(_lib.ttg().ttg_density(op.h, X.h, ptr(occ), r[0], r[1], r[2], n[0], n[1], n[2],
                                 ptr(U[0]), ptr(U[1]), ptr(U[2]), ptr(rho)), "ttg_density")
    return rho.reshape(n[2], n[1], n[0])


def hartree(alpha, omega, G, quad, Uq, grids):
    """Kernel-expansion Hartree potential (see include/ttg.h: ttg_hartree).

    G: (rz, ry, rx) array (x fastest in memory); quad = [(xq, wq)]*3 quadrature
    points and J*w weights; Uq = [(nq, r)]*3 factor values at the quadrature
    points; grids = [x, y, z] target points.  Returns V as (nz, ny, nx) and the
    device time of the contraction launches in ms."""
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    G = np.ascontiguousarray(G, dtype=np.float64)
    rz, ry, rx = G.shape
    q = [(np.ascontiguousarray(a, np.float64), np.ascontiguousarray(w, np.float64)) for a, w in quad]
    U = [np.asfortranarray(u, dtype=np.float64) for u in Uq]
    g = [np.ascontiguousarray(x, np.float64) for x in grids]
    nx, ny, nz = (x.size for x in g)
    V = np.zeros(nx * ny * nz)
    ms = ctypes.c_float()
    check(_lib.ttg().ttg_hartree(alpha.size, ptr(alpha), ptr(omega), rx, ry, rz, ptr(G),
                                 q[0][0].size, q[1][0].size, q[2][0].size,
                                 ptr(q[0][0]), ptr(q[1][0]), ptr(q[2][0]),
                                 ptr(q[0][1]), ptr(q[1][1]), ptr(q[2][1]),
                                 ptr(U[0]), ptr(U[1]), ptr(U[2]), nx, ny, nz,
                                 ptr(g[0]), ptr(g[1]), ptr(g[2]), ptr(V), ctypes.byref(ms)),
          "ttg_hartree")
    return V.reshape(nz, ny, nx), ms.value


def hartree_energy(alpha, omega, G, quad, Uq):
    """1/2 int rho V_H(rho) of a Tucker density on its quadrature grid, FP64
    (see include/ttg.h: ttg_hartree_energy).  G: (rz, ry, rx); quad and Uq as
    for hartree()."""
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    G = np.ascontiguousarray(G, dtype=np.float64)
    rz, ry, rx = G.shape
    q = [(np.ascontiguousarray(a, np.float64), np.ascontiguousarray(w, np.float64)) for a, w in quad]
    U = [np.asfortranarray(u, dtype=np.float64) for u in Uq]
    ranks = np.array([rx, ry, rz], np.int32)
    nq = np.array([q[d][0].size for d in range(3)], np.int32)
    e = ctypes.c_double()
    check(_lib.ttg().ttg_hartree_energy(alpha.size, ptr(alpha), ptr(omega), ptr(ranks), ptr(G),
                                        ptr(nq), ptr(q[0][0]), ptr(q[1][0]), ptr(q[2][0]),
                                        ptr(q[0][1]), ptr(q[1][1]), ptr(q[2][1]),
                                        ptr(U[0]), ptr(U[1]), ptr(U[2]), ctypes.byref(e)),
          "ttg_hartree_energy")
    return e.value
