"""Run a few hot-path launches of one workload, for profilers.

    python -m ttdft_public_gb300.profile_workload --workload atoms64 \
        --prec fp32,bf16 --degrees 1 [--rr] [--states K]
    python -m ttdft_public_gb300.profile_workload --workload atoms64 --scf 1 \
        [--filter mixed] [--mix-alpha 0.1] [--history 10]
    python -m ttdft_public_gb300.profile_workload --hartree 3
    python -m ttdft_public_gb300.profile_workload --gram 64000,256,3

Builds the workload's operator, uploads a random block and runs `degrees`
filter degrees per listed precision (one fused SpMM launch each) and, with
--rr, one Rayleigh-Ritz projection (the df64 SpMM, Gram and eigensolve).  Few
launches and no timing loop, so that an ncu capture of it stays small.  With
--scf N it runs N iterations of the SCF loop instead (for launch lists),
with --hartree N N evaluations of the standalone Hartree contraction."""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from ttdft_public_gb300 import api, system  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="atoms8", choices=sorted(system.CONFIGS))
    ap.add_argument("--prec", default="fp32,bf16")
    ap.add_argument("--degrees", type=int, default=1)
    ap.add_argument("--rr", action="store_true")
    ap.add_argument("--scf", type=int, default=0)
    ap.add_argument("--filter", default="mixed", choices=("fp64", "fp32", "mixed"))
    ap.add_argument("--mix-alpha", type=float, default=0.1,
                    help="Anderson mixing parameter of --scf (the bench's 64-atom setting)")
    ap.add_argument("--history", type=int, default=10, help="Anderson history of --scf")
    ap.add_argument("--states", type=int, default=0, help="block width (default: the workload's)")
    ap.add_argument("--gram", default="",
                    help="instead: N,K,reps: X^T Y of two random N x K blocks (ttg_gram, the FP64 "
                         "tensor-core GEMM) on an identity operator, reps times")
    ap.add_argument("--hartree", type=int, default=0,
                    help="instead: N evaluations of the 35-term Hartree contraction on the "
                         "standalone workload (core 60^3, 360 points per direction)")
    args = ap.parse_args()
    if args.gram:
        import ctypes
        import time
        from ttdft_public_gb300 import _lib
        n, k, reps = (int(x) for x in args.gram.split(","))
        H = system.Csr(n, n, np.arange(n + 1, dtype=np.int64), np.arange(n, dtype=np.int32),
                       np.ones(n))
        op = api.Operator(api.ProjectHamiltonianSparse(H), k)
        rng = np.random.default_rng(0)
        X = api.Mat(op, k, rng.standard_normal((n, k)))
        Y = api.Mat(op, k, rng.standard_normal((n, k)))
        S = np.zeros((k, k), order="F")
        for _ in range(reps):
            t = time.perf_counter()
            assert _lib.ttg().ttg_gram(op.h, X.h, Y.h, ctypes.c_void_p(S.ctypes.data)) == 0
            print(f"gram {n} x {k}: {(time.perf_counter() - t) * 1e3:.2f} ms")
        return
    if args.hartree:
        case = system.hartree_blob_case()
        for _ in range(args.hartree):
            V, ms = api.hartree(*case)
            print(f"hartree contractions {ms:.3f} ms")
        return
    s = system.build_system(system.CONFIGS[args.workload],
                            cache_dir=os.environ.get("TTG_CACHE"))
    if args.scf:
        from ttdft_public_gb300 import scf
        res = scf.Scf(s, scf.ScfConfig(max_iter=args.scf, filter=args.filter,
                                       mix_alpha=args.mix_alpha, history=args.history)).run()
        for h in res["history"]:
            print("iter", h["iter"], "energy", h["energy"], "s", round(h["s"], 3),
                  {k: round(v, 3) for k, v in h["phases"].items()})
        return
    k = args.states or s.spec.n_states
    op = api.Operator(api.ProjectHamiltonianSparse.from_system(s), k)
    X = api.Mat(op, k, np.random.default_rng(0).standard_normal((s.N, k)))
    ax = api.AX(1, k)
    ax.op = op
    lo, hi = -0.5, 20.0
    for p in args.prec.split(","):
        api.ChebyShevFilter(api.sched(p)).computeFilteredSubspace(None, ax, X, s.N, args.degrees,
                                                                 0.0, hi, lo)
    if args.rr:
        api.MultTM().orth(X)
        api.rayleigh_ritz(op, X, rotate=False)
    op.sync()
    print("profile_workload done:", op.info())


if __name__ == "__main__":
    main()
