"""Learned correction to the superposition-of-atomic-densities initial guess.

The reference starts every SCF from a superposition of radial atomic
densities (InitialGuess::initialize_rho, dft/InitialGuess.cc:573-681,
normalised at main.cc:674-680).  Here a small network predicts, per atom, the
coefficients of a correction density built from radial Gaussians centred on
the atom,

    rho_0 = | rho_SAD + sum_a sum_p c_ap exp(-|r - R_a|^2 / w_p^2) |,
    c_a = MLP(D_a),

renormalised to N_e, where D_a are pairwise Gaussian radial descriptors of
the atom's neighbourhood (32 bases, cutoff 8 bohr).  Every term is separable,
so the correction is added on the quadrature grid by the CP-sum kernel.  The
superposition guess stays the fallback (no model file, or guess="sad").

Training data come from the plain method itself: SCF runs from the
superposition guess on seeded random configurations at the 64-atom system's
atom density; for each converged density the per-atom coefficients that best
fit rho_conv - rho_SAD (weighted least squares on the quadrature grid, a small
ridge term) are the regression targets.  The network is trained by the CUDA
kernels of csrc/mlp.cu (forward, backward, Adam).

    python -m ttdft_public_gb300.learned generate --configs 40 --atoms 16 --out DATA.npz
    python -m ttdft_public_gb300.learned train --data DATA.npz [--out MODEL.npz]
    python -m ttdft_public_gb300.learned evaluate --configs 3 --atoms 64 --seed 7001 --out EVAL.jsonl
"""
from __future__ import annotations

import argparse
import ctypes
import dataclasses
import math
import os
import time

import numpy as np

from . import _lib
from ._lib import check, ptr

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "data", "learned_guess.npz")
DEFAULT_DATA = os.path.join(HERE, "data", "learned_train16.npz")

N_FEATURES = 32
MU0, MU1 = 0.5, 8.0
DMU = (MU1 - MU0) / (N_FEATURES - 1)
ETA = 1.0 / (2.0 * 0.35 ** 2)
RCUT = 8.0
WIDTHS = np.geomspace(0.4, 3.2, 6)          # radial Gaussians of the correction
SIZES = [N_FEATURES, 32, 32, len(WIDTHS)]
RIDGE = 1e-6


# ---- descriptors and the network (CUDA) -----------------------------------
def descriptors(atoms) -> np.ndarray:
    pos = np.ascontiguousarray(atoms, dtype=np.float64)
    out = np.zeros((pos.shape[0], N_FEATURES), np.float32)
    check(_lib.ttg().ttg_atom_descriptors(pos.shape[0], ptr(pos), N_FEATURES, MU0, DMU, ETA, RCUT,
                                          ptr(out)), "ttg_atom_descriptors")
    return out


def n_params(sizes=SIZES) -> int:
    return int(sum(i * o + o for i, o in zip(sizes[:-1], sizes[1:])))


def init_params(sizes=SIZES, seed=0) -> np.ndarray:
    """Glorot-uniform weights, zero biases, packed per layer (W row-major, b)."""
    rng = np.random.default_rng(seed)
    out = []
    for i, o in zip(sizes[:-1], sizes[1:]):
        lim = math.sqrt(6.0 / (i + o))
        out.append(rng.uniform(-lim, lim, i * o))
        out.append(np.zeros(o))
    return np.concatenate(out).astype(np.float32)


class Net:
    """Handle on a ttg_mlp (the network's parameters live on the device)."""

    def __init__(self, sizes=SIZES, params=None):
        self.sizes = list(sizes)
        self.lib = _lib.ttg()
        h = ctypes.c_void_p()
        arr = np.array(self.sizes, np.int32)
        check(self.lib.ttg_mlp_create(len(self.sizes) - 1, ptr(arr), ctypes.byref(h)),
              "ttg_mlp_create")
        self.h = h
        self.n = int(self.lib.ttg_mlp_num_params(h))
        self.set(init_params(self.sizes) if params is None else params)

    def set(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n
        check(self.lib.ttg_mlp_set_params(self.h, ptr(p)), "ttg_mlp_set_params")

    def get(self) -> np.ndarray:
        p = np.zeros(self.n, np.float32)
        check(self.lib.ttg_mlp_get_params(self.h, ptr(p)), "ttg_mlp_get_params")
        return p

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], self.sizes[-1]), np.float32)
        check(self.lib.ttg_mlp_forward(self.h, ptr(x), x.shape[0], ptr(y)), "ttg_mlp_forward")
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.n, np.float32)
        loss = ctypes.c_float()
        check(self.lib.ttg_mlp_gradients(self.h, ptr(x), ptr(t), x.shape[0], ptr(g),
                                         ctypes.byref(loss)), "ttg_mlp_gradients")
        return loss.value, g

    def train(self, x, t, epochs, batch=64, lr=1e-3, weight_decay=1e-4, seed=0) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        hist = np.zeros(epochs, np.float32)
        check(self.lib.ttg_mlp_train(self.h, ptr(x), ptr(t), x.shape[0], epochs, batch, lr,
                                     weight_decay, seed, ptr(hist)), "ttg_mlp_train")
        return hist

    def close(self):
        if getattr(self, "h", None):
            self.lib.ttg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class Model:
    params: np.ndarray
    x_mean: np.ndarray
    x_std: np.ndarray
    y_scale: np.ndarray
    sizes: list
    info: dict

    def save(self, path):
        np.savez(path, params=self.params, x_mean=self.x_mean, x_std=self.x_std,
                 y_scale=self.y_scale, sizes=np.array(self.sizes), widths=WIDTHS,
                 info=np.array(repr(self.info)))

    @staticmethod
    def load(path) -> "Model":
        z = np.load(path, allow_pickle=False)
        if not np.allclose(z["widths"], WIDTHS):
            raise ValueError(f"{path}: radial widths differ from this build's")
        return Model(z["params"].astype(np.float32), z["x_mean"], z["x_std"], z["y_scale"],
                     [int(v) for v in z["sizes"]], {"repr": str(z["info"])})

    def predict(self, atoms) -> np.ndarray:
        """Correction coefficients (n_atoms x len(WIDTHS)) for a configuration."""
        d = descriptors(atoms)
        net = Net(self.sizes, self.params)
        try:
            y = net.forward((d - self.x_mean) / self.x_std)
        finally:
            net.close()
        return y.astype(np.float64) * self.y_scale


def load_default(path=DEFAULT_MODEL):
    return Model.load(path) if os.path.exists(path) else None


# ---- the correction density ------------------------------------------------
def correction_factors(atoms, grids):
    """1-D factors of the separable correction terms, term j = (atom a, width p)
    ordered atom-major: fx[j] = exp(-(x - X_a)^2 / w_p^2), etc."""
    f = []
    for d in range(3):
        x = np.asarray(grids[d])
        f.append(np.stack([np.exp(-(x - a[d]) ** 2 / (w * w)) for a in atoms for w in WIDTHS]))
    return f


def fit_targets(atoms, grids, weights, rho_diff):
    """Coefficients c (n_atoms x P) minimising || rho_diff - sum_j c_j g_j ||_W
    (W = product quadrature weights, rho_diff as (nz, ny, nx)), with a small
    ridge term relative to the Gram diagonal."""
    F = correction_factors(atoms, grids)
    G = np.ones((F[0].shape[0],) * 2)
    for d in range(3):
        G *= (F[d] * weights[d]) @ F[d].T
    Fw = [F[d] * weights[d] for d in range(3)]
    t1 = np.einsum("zyx,jx->zyj", rho_diff, Fw[0], optimize=True)
    t2 = np.einsum("zyj,jy->zj", t1, Fw[1], optimize=True)
    b = np.einsum("zj,jz->j", t2, Fw[2], optimize=True)
    A = G + RIDGE * np.mean(np.diag(G)) * np.eye(G.shape[0])
    c = np.linalg.solve(A, b)
    return c.reshape(len(atoms), len(WIDTHS))


# ---- data generation and training -----------------------------------------
def training_spec(n_atoms, seed):
    """A configuration at the 64-atom system's atom density and resolution."""
    from . import system
    ref = system.CONFIGS["atoms64"]
    box = ref.box * (n_atoms / ref.n_atoms) ** (1.0 / 3.0)
    return dataclasses.replace(ref, name=f"train{n_atoms}", n_atoms=n_atoms, box=round(box, 3),
                               n_el=int(round(ref.n_el * box / ref.box)),
                               rank=int(round(ref.rank * box / ref.box)),
                               n_states=int(round(ref.n_states * n_atoms / ref.n_atoms)),
                               seed=seed)


def generate(n_configs, n_atoms, seed0, out, filt="mixed", log=print):
    """Plain SCF (superposition guess) on seeded configurations; stores the
    descriptors and fitted correction coefficients of every atom."""
    from . import scf, system
    X, Y, meta = [], [], []
    for i in range(n_configs):
        t0 = time.time()
        spec = training_spec(n_atoms, seed0 + i)
        s = system.build_system(spec)
        g = scf.Scf(s, scf.ScfConfig(filter=filt, mix_alpha=0.1, history=10, max_iter=60))
        rho_sad = g.initial_density().cpu().numpy()
        res = g.run()
        rho = g.rho.cpu().numpy()
        q = [b.fem.nq for b in s.basis]
        grids = [b.fem.xq for b in s.basis]
        wts = [b.fem.wJ for b in s.basis]
        diff = (rho - rho_sad).reshape(q[2], q[1], q[0])
        c = fit_targets(s.atoms, grids, wts, diff)
        X.append(descriptors(s.atoms))
        Y.append(c)
        meta.append((spec.seed, res["iterations"], float(res["converged"]), res["energy"]))
        g.close()
        log(f"config {i}: seed {spec.seed} iterations {res['iterations']} converged "
            f"{res['converged']} E {res['energy']:.6f} ({time.time() - t0:.1f} s)", flush=True)
    np.savez(out, x=np.concatenate(X), y=np.concatenate(Y), meta=np.array(meta, np.float64),
             n_atoms=n_atoms)


def evaluate(n_configs, n_atoms, seed0, out, filt="mixed", log=print):
    """Held-out check of the learned guess: on seeded configurations of
    n_atoms at the 64-atom system's density and resolution (seeds outside
    the training set's), one SCF from the superposition guess and one from
    the learned guess, to the same convergence test; one JSON line per
    configuration, written as each finishes: iterations, wall time, energies
    and start-density errors of both runs."""
    import json
    from . import scf, system
    with open(out, "a") as f:
        for i in range(n_configs):
            spec = training_spec(n_atoms, seed0 + i)
            s = system.build_system(spec)
            row = {"seed": spec.seed, "n_atoms": n_atoms, "N": s.N, "states": spec.n_states}
            for guess in ("sad", "learned"):
                g = scf.Scf(s, scf.ScfConfig(filter=filt, mix_alpha=0.1, history=10,
                                             max_iter=60, guess=guess))
                t0 = time.time()
                res = g.run()
                row[guess] = {"s": round(time.time() - t0, 3), "iterations": res["iterations"],
                              "converged": bool(res["converged"]), "energy_ha": float(res["energy"]),
                              "start_density_error": round(float(g.start_error()), 5),
                              "guess_used": g.guess_used}
                g.close()
                del g
            row["de_atom"] = abs(row["learned"]["energy_ha"] - row["sad"]["energy_ha"]) / n_atoms
            f.write(json.dumps(row) + "\n")
            f.flush()
            log(json.dumps(row), flush=True)


def train(data=DEFAULT_DATA, out=DEFAULT_MODEL, epochs=3000, batch=64, lr=2e-3,
          weight_decay=1e-3, val_frac=0.2, seed=0, chunk=50, log=print):
    """Minibatch Adam on the GPU kernels; the parameters with the lowest
    validation error (checked every `chunk` epochs on held-out
    configurations) are kept."""
    z = np.load(data)
    x, y = z["x"].astype(np.float64), z["y"].astype(np.float64)
    n_at = int(z["n_atoms"])
    n_cfg = x.shape[0] // n_at
    rng = np.random.default_rng(seed)
    order = rng.permutation(n_cfg)
    n_val = max(1, int(round(val_frac * n_cfg)))
    val_cfg, tr_cfg = order[:n_val], order[n_val:]

    def rows(cfgs):
        return np.concatenate([np.arange(c * n_at, (c + 1) * n_at) for c in cfgs])

    itr, iva = rows(tr_cfg), rows(val_cfg)
    # features that barely vary (neighbour shells closer than the minimum
    # separation) are not blown up by the standardisation
    x_mean, x_std = x[itr].mean(0), x[itr].std(0)
    x_std = np.maximum(x_std, 0.05 * x_std.max())
    y_scale = y[itr].std(0) + 1e-12
    xn = ((x - x_mean) / x_std).astype(np.float32)
    yn = (y / y_scale).astype(np.float32)
    net = Net(SIZES)
    best = (np.inf, None, 0)
    hist = []
    try:
        for c in range(max(1, epochs // chunk)):
            hist.extend(net.train(xn[itr], yn[itr], chunk, batch=batch, lr=lr,
                                  weight_decay=weight_decay, seed=seed + c))
            v = float(np.mean((net.forward(xn[iva]) - yn[iva]) ** 2))
            if v < best[0]:
                best = (v, net.get(), (c + 1) * chunk)
    finally:
        net.close()
    val_mse, params, best_epoch = best
    base_mse = float(np.mean((yn[iva] - yn[itr].mean(0)) ** 2))
    info = {"train_configs": len(tr_cfg), "val_configs": len(val_cfg), "atoms": n_at,
            "epochs": len(hist), "best_epoch": best_epoch,
            "train_mse": float(hist[-1]) / SIZES[-1], "val_mse": val_mse,
            "val_mse_of_mean_predictor": base_mse}
    m = Model(params, x_mean, x_std, y_scale, SIZES, info)
    if out:
        m.save(out)
    log(f"trained: {info}")
    return m, info


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("generate")
    g.add_argument("--configs", type=int, default=40)
    g.add_argument("--atoms", type=int, default=16)
    g.add_argument("--seed", type=int, default=5000)
    g.add_argument("--filter", default="mixed")
    g.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", default=DEFAULT_DATA)
    t.add_argument("--out", default=DEFAULT_MODEL)
    t.add_argument("--epochs", type=int, default=3000)
    e = sub.add_parser("evaluate")
    e.add_argument("--configs", type=int, default=3)
    e.add_argument("--atoms", type=int, default=64)
    e.add_argument("--seed", type=int, default=7001)
    e.add_argument("--filter", default="mixed")
    e.add_argument("--out", required=True)
    a = ap.parse_args()
    if a.cmd == "generate":
        generate(a.configs, a.atoms, a.seed, a.out, a.filter)
    elif a.cmd == "evaluate":
        evaluate(a.configs, a.atoms, a.seed, a.out, a.filter)
    else:
        train(a.data, a.out, epochs=a.epochs)


if __name__ == "__main__":
    main()
