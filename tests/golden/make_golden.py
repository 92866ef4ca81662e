"""Writes tests/golden/tiny.npz: outputs of the FP64 oracle on the seeded
2-atom system (system.small_spec()) and the 2-atom SCF system, frozen as
regression anchors for the oracle and the CUDA path.

The reference ships no tests or golden vectors and cannot be built here, so
these fixtures are generated by this repository's oracle; they pin the
oracle against later changes and give the GPU tests fixed targets.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import scf as oscf  # noqa: E402
from ttdft_public_gb300 import scf, system  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tiny.npz")

# parameters of every fixture, also read by the tests
FILTER = dict(m=8, a=0.0, b=30.0, a0=-0.5)
LANCZOS_ITERS = 20
PASSES = 6


def scf_spec():
    return system.small_spec(name="scf", n_atoms=2, box=10.0, n_el=16, rank=8, n_states=12,
                             degree=12, seed=3)


def scf_config():
    return scf.ScfConfig(max_iter=25, restarts_first=6, restarts_other=4)


def inputs(s):
    k = s.spec.n_states
    X0 = np.random.default_rng(0).standard_normal((s.N, k))
    v0 = np.random.default_rng(1).uniform(0, 1, s.N)
    return X0, v0


def compute():
    s = system.build_system(system.small_spec())
    X0, v0 = inputs(s)
    out = {"fingerprint": np.array([s.N, s.H.row_ptr[-1], s.H.val.sum(), np.abs(s.C.val).sum()])}
    out["filter_prev"] = oracle.cheb_filter(s, X0, FILTER["m"], FILTER["a"], FILTER["b"],
                                            FILTER["a0"], return_prev=True)
    out["filter_m"] = oracle.cheb_filter(s, X0, FILTER["m"], FILTER["a"], FILTER["b"],
                                         FILTER["a0"], return_prev=False)
    al, be = oracle.lanczos_T(s, v0, LANCZOS_ITERS)
    out["lanczos_alpha"], out["lanczos_beta"] = al, be
    out["lanczos_bounds"] = np.array(oracle.lanczos_bounds(s, v0, LANCZOS_ITERS))
    up, lo = out["lanczos_bounds"]
    X, a, a0 = X0, 0.0, lo
    for _ in range(PASSES):
        w, _, X = oracle.chfsi_pass(s, X, s.spec.degree, a, up, a0)
        a0, a = w[0], w[-1]
    out["chfsi_eigenvalues"] = w
    rho = np.linspace(1e-5, 0.5, 64)
    out["lda_rho"] = rho
    out["lda_v"], out["lda_e"] = oscf.lda(rho)
    ss = system.build_system(scf_spec())
    run = oscf.OracleScf(ss, scf_config()).run()
    out["scf_energies"] = np.array([h["energy"] for h in run["history"]])
    return out


if __name__ == "__main__":
    np.savez(OUT, **compute())
    print("wrote", OUT)
