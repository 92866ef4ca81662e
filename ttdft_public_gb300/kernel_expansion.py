"""Gaussian expansion of the Coulomb kernel, 1/r ~ sum_k w_k exp(-a_k r^2).

The reference reads its exponents and weights from files fitted to
1/sqrt(x) on [1, 1e8] and rescales them by A^2 (dft/KSDFTPotential.cc:
273-284); with its A^2 = 4.04e-5 they span r in [A, 1e4 A] ~ [6e-3, 64] bohr.
Here 35 terms are fitted to 1/r on [5e-3, 64] bohr (max relative error
1.15e-5) and stored in data/coulomb_expansion_35.txt.  All weights are
positive, so the expansion sums without cancellation, which the FP32
tensor-core contraction needs.

The fit (run `python -m ttdft_public_gb300.kernel_expansion --fit`): start
from the trapezoidal rule of 1/r = (2/sqrt(pi)) int exp(-r^2 t^2) dt in
s = log t, then optimise log-exponents and log-weights by nonlinear least
squares on log-spaced r, reweighting the residuals towards their maxima.
"""
from __future__ import annotations

import functools
import math
import os

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                     "coulomb_expansion_35.txt")
RMIN, RMAX = 5e-3, 64.0


@functools.lru_cache(maxsize=1)
def coulomb_expansion():
    """(alpha, omega): the stored 35-term expansion."""
    t = np.loadtxt(_DATA)
    return t[:, 0].copy(), t[:, 1].copy()


def expansion_error(alpha, omega, rmin=RMIN, rmax=RMAX):
    r = np.geomspace(rmin, rmax, 20000)
    approx = np.exp(-np.outer(r * r, alpha)) @ omega
    return float(np.max(np.abs(approx * r - 1.0)))


def fit(K=35, rmin=RMIN, rmax=RMAX, rounds=25, seconds=600.0):
    """Regenerates the table (scipy; a few minutes)."""
    import time

    import scipy.optimize
    s = np.linspace(math.log(2.9e-4 / rmax), math.log(1.8 / rmin), K)
    h = s[1] - s[0]
    p = np.concatenate([s, np.log(2.0 / math.sqrt(math.pi) * h) + s])
    r = np.geomspace(rmin, rmax, 1500)

    def res(q, wt):
        return ((np.exp(-np.outer(r * r, np.exp(2 * q[:K]))) @ np.exp(q[K:])) * r - 1.0) * wt

    def jac(q, wt):
        a, w = np.exp(2 * q[:K]), np.exp(q[K:])
        E = np.exp(-np.outer(r * r, a))
        Js = (E * (-(r * r))[:, None] * (2 * a * w)[None, :]) * r[:, None]
        return np.hstack([Js, E * w[None, :] * r[:, None]]) * wt[:, None]

    wt = np.ones_like(r)
    best = None
    t0 = time.time()
    for _ in range(rounds):
        p = scipy.optimize.least_squares(res, p, jac=jac, args=(wt,), method="trf", max_nfev=300,
                                         xtol=1e-15, ftol=1e-15, gtol=1e-15).x
        a, w = np.exp(2 * p[:K]), np.exp(p[K:])
        e = expansion_error(a, w, rmin, rmax)
        if best is None or e < best[0]:
            best = (e, a, w)
        f = np.abs(res(p, np.ones_like(r)))
        wt = wt * (1.0 + 4.0 * f / f.max())
        wt /= wt.mean()
        if time.time() - t0 > seconds:
            break
    return best


if __name__ == "__main__":
    import sys
    if "--fit" in sys.argv:
        e, a, w = fit()
        o = np.argsort(a)
        with open(_DATA, "w") as f:
            f.write(f"# 1/r ~ sum_k omega_k exp(-alpha_k r^2), r in [{RMIN:g}, {RMAX:g}] bohr, "
                    f"max relative error {e:.3g}\n")
            f.write("# made by: python -m ttdft_public_gb300.kernel_expansion --fit\n")
            f.write("# alpha_k (bohr^-2)          omega_k\n")
            for i in o:
                f.write(f"{a[i]:.17e} {w[i]:.17e}\n")
    a, w = coulomb_expansion()
    print(len(a), "terms, max relative error", expansion_error(a, w))
