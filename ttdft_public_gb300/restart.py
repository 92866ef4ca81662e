"""The reference's restart tree: what an SCF run leaves on disk after every
iteration so that a later run can resume it.

Layout (main.cc:690-697, dft/AndersonMixing.cc:53-143, 376-443):

  <root>/rank_<rx>_<ry>_<rz>/wfn/wfn_proc0          the eigenvector block X
  <root>/rank_<rx>_<ry>_<rz>/wfn/cheby_bounds.txt   six bounds and energies
  <root>/rank_<rx>_<ry>_<rz>/rho/history_scf.txt    SCF iterations kept, one per line
  <root>/rank_<rx>_<ry>_<rz>/rho/rho_<kind>/rho_<kind>_scf<i>_proc0
        kind = quad_in, quad_out (the Anderson history on the quadrature
        grid) and nodal_out (the output density on the nodes)

Binary files are raw FP64 arrays with no header, big-endian, as PETSc's
PetscBinaryWrite writes them (main.cc:1167-1173, AndersonMixing.cc:465-479):
X is the N x k block column by column (the PETSc dense layout), densities are
x-fastest fields.  cheby_bounds.txt holds, tab-separated in %.16e, the upper
bound of the unwanted spectrum, the lower bound of the unwanted spectrum, the
lowest wanted eigenvalue, the relative error of the upper bound, the
occupied-orbital energy and the previous total energy (main.cc:1150-1157).

The reference also keeps the nodal input densities; the mixing here works on
the quadrature grid only, so their history is not written.
"""
from __future__ import annotations

import os

import numpy as np

BOUNDS = ("upper", "lower_unwanted", "lower_wanted", "err_upper", "occ_energy", "e_old")
KINDS = ("quad_in", "quad_out", "nodal_out")


def tree(root: str, ranks) -> str:
    return os.path.join(root, "rank_%d_%d_%d" % tuple(int(r) for r in ranks))


def _paths(root, ranks):
    t = tree(root, ranks)
    return os.path.join(t, "wfn"), os.path.join(t, "rho")


def write_array(path: str, a: np.ndarray, order: str = "C") -> None:
    np.asarray(a, dtype=np.float64).ravel(order=order).astype(">f8").tofile(path)


def read_array(path: str, n: int) -> np.ndarray:
    a = np.fromfile(path, dtype=">f8")
    if a.size != n:
        raise ValueError(f"{path}: {a.size} values, expected {n}")
    return a.astype(np.float64)


def write_bounds(root, ranks, bounds: dict) -> None:
    wfn, _ = _paths(root, ranks)
    os.makedirs(wfn, exist_ok=True)
    with open(os.path.join(wfn, "cheby_bounds.txt"), "w") as f:
        f.write("\t".join("%.16e" % float(bounds[k]) for k in BOUNDS))


def read_bounds(root, ranks) -> dict:
    wfn, _ = _paths(root, ranks)
    with open(os.path.join(wfn, "cheby_bounds.txt")) as f:
        vals = [float(x) for x in f.read().split()]
    if len(vals) != len(BOUNDS):
        raise ValueError("cheby_bounds.txt: expected six values")
    return dict(zip(BOUNDS, vals))


def write_wfn(root, ranks, X: np.ndarray) -> None:
    """X: N x k (the block, any memory order); written column by column."""
    wfn, _ = _paths(root, ranks)
    os.makedirs(wfn, exist_ok=True)
    write_array(os.path.join(wfn, "wfn_proc0"), X, order="F")


def read_wfn(root, ranks, n: int, k: int) -> np.ndarray:
    wfn, _ = _paths(root, ranks)
    return read_array(os.path.join(wfn, "wfn_proc0"), n * k).reshape((n, k), order="F")


def rho_file(root, ranks, kind: str, scf: int) -> str:
    _, rho = _paths(root, ranks)
    return os.path.join(rho, "rho_" + kind, "rho_%s_scf%d_proc0" % (kind, scf))


def write_history_entry(root, ranks, scf: int, fields: dict, keep: int) -> list[int]:
    """Writes this iteration's densities (kind -> x-fastest array), removes
    the files of iterations that fell out of a history of `keep`, and rewrites
    history_scf.txt (AndersonMixing.cc:376-443).  Returns the kept list."""
    _, rho = _paths(root, ranks)
    for kind, a in fields.items():
        os.makedirs(os.path.join(rho, "rho_" + kind), exist_ok=True)
        write_array(rho_file(root, ranks, kind, scf), a)
    kept = read_history(root, ranks) + [scf]
    kept = sorted(set(kept))
    while len(kept) > keep:
        old = kept.pop(0)
        for kind in KINDS:
            p = rho_file(root, ranks, kind, old)
            if os.path.exists(p):
                os.remove(p)
    with open(os.path.join(rho, "history_scf.txt"), "w") as f:
        f.write("".join("%d\n" % i for i in kept))
    return kept


def read_history(root, ranks) -> list[int]:
    _, rho = _paths(root, ranks)
    p = os.path.join(rho, "history_scf.txt")
    if not os.path.exists(p):
        return []
    with open(p) as f:
        return [int(x) for x in f.read().split()]
