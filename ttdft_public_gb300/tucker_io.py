"""Tucker files of an electron density, in the reference's on-disk format.

The reference writes the converged nodal density as a Tucker tensor
(write_out_rho, main.cc:1528-1632) and can start an SCF from such files
(InitialGuess::initialize_rho_tucker, dft/InitialGuess.cc:764-904, with
read_in_factor_matrices and construct_local_factor_matrices at
dft/InitialGuess.cc:1211-1307).  The format:

- core file: one line "r0 r1 r2", then the r0 r1 r2 core values, one per
  line, x fastest (%.18e);
- one factor file per direction: a line "n_nodes rank", a line with the
  n_nodes nodal coordinates, then `rank` lines, line r holding column r of
  the factor at those nodes (tab-separated, %.18e).

Written files are named rank_<r>_core and rank_<r>_factor_{x,y,z}, where <r>
is the calculation's basis rank in that direction (main.cc:1571, 1619-1631);
the reader takes tucker_input_core and tucker_input_factor_{x,y,z}.  On
reading, each factor column becomes the cubic spline through its nodal
values with zero first derivative at both ends (ALGLIB spline1dbuildcubic
with boundary types 1 and values 0, InitialGuess.cc:1277-1284), evaluated
wherever the density is wanted: the nodes or the quadrature points.  The
spline here is this module's own restatement of the clamped cubic spline.
"""
from __future__ import annotations

import math
import os

import numpy as np
import scipy.linalg

CORE_IN = "tucker_input_core"
FACTOR_IN = ("tucker_input_factor_x", "tucker_input_factor_y", "tucker_input_factor_z")


def output_ranks(n_nodes) -> list[int]:
    """Tucker ranks of the written density (main.cc:1543-1557):
    int(100 log n / log 250) per direction, or int(0.6 n) when that is not
    below the node count."""
    out = []
    for n in n_nodes:
        r = int(100 * math.log(n) / math.log(250))
        if r >= n:
            r = int(n * 0.6)
        out.append(r)
    return out


def write_core(path: str, core: np.ndarray) -> None:
    """core: (r0, r1, r2) array; written with x (axis 0) fastest."""
    r0, r1, r2 = core.shape
    with open(path, "w") as f:
        f.write(f"{r0} {r1} {r2}\n")
        for v in np.asarray(core, np.float64).reshape(-1, order="F"):
            f.write(f"{v:.18e}\n")


def read_core(path: str) -> np.ndarray:
    with open(path) as f:
        tok = f.read().split()
    r = [int(t) for t in tok[:3]]
    vals = np.array([float(t) for t in tok[3:3 + r[0] * r[1] * r[2]]], np.float64)
    if vals.size != r[0] * r[1] * r[2]:
        raise ValueError(f"{path}: {vals.size} core values, expected {r[0] * r[1] * r[2]}")
    return vals.reshape(r, order="F")


def write_factor(path: str, coords: np.ndarray, U: np.ndarray) -> None:
    """U: (n_nodes, rank) factor at the nodal coordinates."""
    n, rank = U.shape
    if len(coords) != n:
        raise ValueError("one coordinate per factor row")
    with open(path, "w") as f:
        f.write(f"{n} {rank}\n")
        f.write("".join(f"{x:.18e}\t" for x in coords) + "\n")
        for r in range(rank):
            f.write("".join(f"{v:.18e}\t" for v in U[:, r]) + "\n")


def read_factor(path: str) -> tuple[np.ndarray, np.ndarray]:
    """(coords (n,), U (n, rank))."""
    with open(path) as f:
        n, rank = (int(t) for t in f.readline().split()[:2])
        coords = np.array([float(t) for t in f.readline().split()[:n]], np.float64)
        U = np.empty((n, rank))
        for r in range(rank):
            row = [float(t) for t in f.readline().split()[:n]]
            if len(row) != n:
                raise ValueError(f"{path}: factor column {r} has {len(row)} values, expected {n}")
            U[:, r] = row
    if coords.size != n:
        raise ValueError(f"{path}: {coords.size} coordinates, expected {n}")
    return coords, U


class ClampedCubic:
    """Cubic splines through (x_i, y_i) for every column of y, with s'(x_0) =
    s'(x_n) = 0.  The second derivatives M solve the tridiagonal system
    h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1} =
    6 ((y_{i+1} - y_i) / h_i - (y_i - y_{i-1}) / h_{i-1}), closed by
    2 h_0 M_0 + h_0 M_1 = 6 (y_1 - y_0) / h_0 and
    h_{n-1} M_{n-1} + 2 h_{n-1} M_n = -6 (y_n - y_{n-1}) / h_{n-1}.
    Points outside [x_0, x_n] use the end segments' cubics."""

    def __init__(self, x: np.ndarray, y: np.ndarray):
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        if y.ndim == 1:
            y = y[:, None]
        n = x.size
        if n < 2 or np.any(np.diff(x) <= 0):
            raise ValueError("spline knots must be increasing, at least two")
        h = np.diff(x)
        ab = np.zeros((3, n))          # banded: super, main, sub
        rhs = np.zeros((n, y.shape[1]))
        slope = np.diff(y, axis=0) / h[:, None]
        ab[1, 0], ab[0, 1] = 2 * h[0], h[0]
        rhs[0] = 6 * slope[0]
        for i in range(1, n - 1):
            ab[2, i - 1] = h[i - 1]
            ab[1, i] = 2 * (h[i - 1] + h[i])
            ab[0, i + 1] = h[i]
            rhs[i] = 6 * (slope[i] - slope[i - 1])
        ab[2, n - 2], ab[1, n - 1] = h[n - 2], 2 * h[n - 2]
        rhs[n - 1] = -6 * slope[n - 2]
        self.x, self.y, self.h = x, y, h
        self.M = scipy.linalg.solve_banded((1, 1), ab, rhs)

    def __call__(self, t: np.ndarray) -> np.ndarray:
        t = np.asarray(t, np.float64)
        i = np.clip(np.searchsorted(self.x, t, side="right") - 1, 0, self.x.size - 2)
        h = self.h[i][:, None]
        a = (self.x[i + 1] - t)[:, None]
        b = (t - self.x[i])[:, None]
        Mi, Mj = self.M[i], self.M[i + 1]
        yi, yj = self.y[i], self.y[i + 1]
        return (Mi * a ** 3 + Mj * b ** 3) / (6 * h) + (yi / h - Mi * h / 6) * a + \
            (yj / h - Mj * h / 6) * b


def factors_at(coords: np.ndarray, U: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Factor columns evaluated at t (construct_local_factor_matrices)."""
    return ClampedCubic(coords, U)(t)


def write_density(dirpath: str, core: np.ndarray, coords, factors, basis_ranks) -> list[str]:
    """The files of write_out_rho: rank_<r>_core and rank_<r>_factor_{x,y,z},
    <r> the calculation's basis rank per direction.  core (r0, r1, r2), x
    fastest; factors[d] (n_d, r_d) at the nodal coordinates coords[d]."""
    os.makedirs(dirpath, exist_ok=True)
    names = [os.path.join(dirpath, f"rank_{basis_ranks[0]}_core")]
    write_core(names[0], core)
    for d, ax in enumerate("xyz"):
        names.append(os.path.join(dirpath, f"rank_{basis_ranks[d]}_factor_{ax}"))
        write_factor(names[-1], coords[d], factors[d])
    return names


def read_density(dirpath: str):
    """(core (r0, r1, r2), [(coords_d, U_d)] * 3) from tucker_input_core and
    tucker_input_factor_{x,y,z} in dirpath."""
    core = read_core(os.path.join(dirpath, CORE_IN))
    fac = [read_factor(os.path.join(dirpath, name)) for name in FACTOR_IN]
    for d in range(3):
        if fac[d][1].shape[1] != core.shape[d]:
            raise ValueError(f"factor {d} has rank {fac[d][1].shape[1]}, core {core.shape[d]}")
    return core, fac


def reconstruct(core: np.ndarray, U) -> np.ndarray:
    """core x_1 U0 x_2 U1 x_3 U2, as an (n0, n1, n2) array."""
    return np.einsum("abc,ia,jb,kc->ijk", core, U[0], U[1], U[2], optimize=True)
