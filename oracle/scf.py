"""FP64 CPU restatement of the SCF loop -- TEST INFRASTRUCTURE ONLY.

Same steps, constants and conventions as ttdft_public_gb300/scf.py (which
restates main.cc:846-1522); every grid operation here is numpy/scipy and the
eigensolver path is the C oracle, so this is the checker for the GPU SCF on
small systems.  The Hamiltonian's values are recomputed on the pattern fixed
at the start, as the GPU path does.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.special

import oracle
from ttdft_public_gb300.kernel_expansion import coulomb_expansion
from ttdft_public_gb300.scf import KB_HA_PER_K, ScfConfig, potential_matrices, repulsive_energy
from ttdft_public_gb300.system import Csr


def sthosvd(T, eps, cap):
    """Sequentially truncated HOSVD of an x-fastest tensor given as (n2, n1, n0)
    array: per mode, eigenvectors of the mode Gram matrix, discarding the
    smallest eigenvalues while their sum stays <= eps^2 |T|^2 / 3 (eps 0: the
    rank is the cap, as the fixed-rank STHOSVD of main.cc:952-956)."""
    A = np.transpose(T, (2, 1, 0)).copy()          # (n0, n1, n2): mode d = axis d
    thr = eps * eps * float(np.sum(A * A)) / 3.0
    U = []
    for d in range(3):
        M = np.moveaxis(A, d, 0).reshape(A.shape[d], -1)
        w, V = np.linalg.eigh(M @ M.T)
        disc, r = 0.0, len(w)
        for i in range(len(w)):
            lam = max(w[i], 0.0)
            if disc + lam > thr:
                break
            disc += lam
            r = len(w) - i - 1
        r = max(1, min(r if eps > 0 else len(w), cap))     # eps 0: exactly the cap
        Ud = V[:, ::-1][:, :r]
        U.append(Ud)
        A = np.moveaxis(np.tensordot(Ud.T, np.moveaxis(A, d, 0), axes=(1, 0)), 0, d)
    return A, U                                       # core (r0, r1, r2)


def reconstruct(core, U):
    return np.einsum("abc,ia,jb,lc->lji", core, U[0], U[1], U[2], optimize=True)


def lda(rho):
    """Potential and energy density as ttg_grid_lda (KSDFTPotential.cc:127-267,
    KSDFTEnergyFunctional.cc:27-56, the reference's constants and formulas)."""
    g, b1, b2, A, B, C, D = -0.1423, 1.0529, 0.3334, 0.0311, -0.048, 0.002, -0.0116
    exch_c = -(3.0 / 4.0) * np.cbrt(3.0 / math.pi)
    c0 = np.cbrt(3.0 / (4.0 * math.pi))
    cr = np.cbrt(rho)
    vx = exch_c * (4.0 / 3.0) * cr
    ex = exch_c * rho * cr
    with np.errstate(divide="ignore"):
        rsv = np.cbrt(3.0 / (4.0 * math.pi * rho))
    hi = rsv >= 1.0
    vc = np.empty_like(rho)
    sq = np.sqrt(rsv[hi])
    den = 1.0 + b1 * sq + b2 * rsv[hi]
    vc[hi] = g * (1.0 + 7.0 / 6.0 * b1 * sq + 4.0 / 3.0 * b2 * rsv[hi]) / den ** 2
    lo = ~hi
    lr = np.log(rsv[lo])
    vc[lo] = A * lr + (B - A / 3.0) + 2.0 / 3.0 * C * rsv[lo] * lr + (2 * D - C) * rsv[lo] / 33.0
    rs = c0 / (cr + 1e-12)
    ec = np.where(rs >= 1.0, g / (1.0 + b1 * np.sqrt(rs) + b2 * rs),
                  A * np.log(rs) + B + C * rs * np.log(rs) + D * rs)
    return vx + vc, ex + ec * rho


class OracleScf:
    def __init__(self, sysm, cfg: ScfConfig | None = None, n_states=None, degree=None):
        self.s = sysm
        self.cfg = cfg or ScfConfig()
        spec = sysm.spec
        self.k = n_states or spec.n_states
        self.m = degree or spec.degree
        self.ne = spec.n_electrons
        self.natoms = spec.n_atoms
        b = sysm.basis
        self.xq = [bb.fem.xq for bb in b]
        self.w = [bb.fem.wJ for bb in b]
        self.W = self.w[2][:, None, None] * self.w[1][None, :, None] * self.w[0][None, None, :]
        self.alpha, self.omega = coulomb_expansion()
        # V_loc: Gaussian wells + Gaussian ionic charges (exact erf potential)
        X, Y, Z = np.meshgrid(self.xq[0], self.xq[1], self.xq[2], indexing="ij")
        v = np.zeros(X.shape)
        for a in sysm.atoms:
            d2 = (X - a[0]) ** 2 + (Y - a[1]) ** 2 + (Z - a[2]) ** 2
            v -= spec.z_val * np.exp(-d2 / (2 * spec.sigma ** 2))
            r = np.sqrt(d2)
            with np.errstate(divide="ignore", invalid="ignore"):
                v -= spec.z_val * np.where(r > 1e-10, scipy.special.erf(r / self.cfg.ion_width) / r,
                                           2.0 / (math.sqrt(math.pi) * self.cfg.ion_width))
        self.vloc = np.transpose(v, (2, 1, 0)).copy()          # (z, y, x)
        self.e_nn = repulsive_energy(sysm.atoms, spec.z_val)
        # pattern and 1-D matrices
        H = sysm.H
        self.rows = np.repeat(np.arange(H.n_rows), np.diff(H.row_ptr))
        self.cols = H.col.astype(np.int64)
        r = [bb.r for bb in b]
        self.r = r
        self.I3 = (self.rows % r[0], (self.rows // r[0]) % r[1], self.rows // (r[0] * r[1]))
        self.J3 = (self.cols % r[0], (self.cols // r[0]) % r[1], self.cols // (r[0] * r[1]))
        DX, DY, DZ = (bb.stiffness() for bb in b)
        MX, MY, MZ = (bb.overlap() for bb in b)
        (xi, yi, zi), (xj, yj, zj) = self.I3, self.J3
        self.kin = 0.5 * (DX[xi, xj] * MY[yi, yj] * MZ[zi, zj] + MX[xi, xj] * DY[yi, yj] * MZ[zi, zj]
                          + MX[xi, xj] * MY[yi, yj] * DZ[zi, zj])

    def integrate(self, f, g=None):
        return float(np.sum(f * (1.0 if g is None else g) * self.W))

    def hartree(self, core, U):
        quad = [(self.xq[d], self.w[d]) for d in range(3)]
        return oracle.hartree(self.alpha, self.omega, np.transpose(core, (2, 1, 0)), quad, U,
                              self.xq)

    def initial_density(self):
        spec, w = self.s.spec, self.cfg.sad_width
        rho = oracle.sad_density(self.s.atoms, self.xq, spec.z_val, w)
        return rho * (self.ne / self.integrate(rho))

    def veff_from(self, rho_in):
        core, U = sthosvd(rho_in, self.cfg.rho_eps, self.cfg.rho_rank_cap)
        vxc, _ = lda(rho_in)
        return self.vloc + self.hartree(core, U) + vxc

    def hamiltonian(self, veff):
        core, U = sthosvd(veff, self.cfg.veff_eps, self.cfg.veff_rank_cap)
        P = [potential_matrices(self.s.basis[d], U[d]) for d in range(3)]
        (xi, yi, zi), (xj, yj, zj) = self.I3, self.J3
        # sum_abc core[a,b,c] P0[a,xi,xj] P1[b,yi,yj] P2[c,zi,zj] over the
        # pattern: the (y, z) pair part tabulated once, entries in chunks
        r = self.r
        ypair, yinv = np.unique(yi * r[1] + yj, return_inverse=True)
        zpair, zinv = np.unique(zi * r[2] + zj, return_inverse=True)
        B = P[1][:, ypair // r[1], ypair % r[1]]                 # (rb, ny)
        C = P[2][:, zpair // r[2], zpair % r[2]]                 # (rc, nz)
        Q = np.einsum("abc,bj,ck->jka", core, B, C, optimize=True)
        vals = self.kin.copy()
        step = 1 << 18
        for s0 in range(0, vals.size, step):
            e = slice(s0, s0 + step)
            A = P[0][:, xi[e], xj[e]]                            # (ra, chunk)
            vals[e] += np.einsum("ae,ea->e", A, Q[yinv[e], zinv[e]])
        H = self.s.H
        return Csr(H.n_rows, H.n_cols, H.row_ptr, H.col, vals)

    def density_out(self, X, occ):
        rho_n = oracle.density(X, occ, self.s.basis)
        core, U = sthosvd(rho_n, self.cfg.rho_out_eps, self.cfg.rho_out_rank_cap)
        Uq = [self.s.basis[d].fem.interp_matrix() @ U[d] for d in range(3)]
        return np.abs(reconstruct(core, Uq)), (core, Uq)

    def run(self, max_iter=None):
        cfg = self.cfg
        k, m = self.k, self.m
        kT = KB_HA_PER_K * cfg.temperature
        X = np.random.default_rng(cfg.seed).standard_normal((self.s.N, k))
        v0 = np.random.default_rng(cfg.seed + 1).uniform(0, 1, self.s.N)
        occ_idx = min(int(self.ne / 2.0 + 10), k - 1)
        hist_in, hist_out, history = [], [], []
        upper, err_upper = 1e16, 1e16
        lower_wanted = lower_unwanted = None
        occ_energy, e_old, w = 1e9, None, None
        rho_in = self.initial_density()

        class S:
            pass
        for it in range(max_iter or cfg.max_iter):
            if it > 0:
                rho_in = self.anderson(hist_in, hist_out)
            veff = self.veff_from(rho_in)
            sysH = S()
            sysH.H, sysH.C, sysH.D = self.hamiltonian(veff), self.s.C, self.s.D
            if err_upper > 0.01:
                cur, tmp_lower = oracle.lanczos_bounds(sysH, v0, cfg.lanczos_iter)
                err_upper = (upper - cur) / upper
                upper = cur if err_upper > 0.01 else cur * 1.05
                if it == 0:
                    lower_wanted, lower_unwanted = tmp_lower, 0.0
            if it > 0:
                lower_wanted, lower_unwanted = w[0], w[-1]
            restarts = cfg.restarts_first if it == 0 else cfg.restarts_other
            for _ in range(restarts):
                X = oracle.cheb_filter(sysH, X, m, lower_unwanted, upper, lower_wanted)
                X, st = oracle.cholqr(X)
                w, Q, X = oracle.rayleigh_ritz(sysH, X)
                lower_wanted, lower_unwanted = w[0], w[-1]
                err = abs((w[occ_idx] - occ_energy) / occ_energy)
                occ_energy = w[occ_idx]
                if err < cfg.cheb_tol:
                    break
            mu, occ = oracle.fermi(w, self.ne, kT)
            rho_out, (core, Uq) = self.density_out(X, occ)
            vh_out = self.hartree(core, Uq)
            _, exc = lda(rho_out)
            e_grid = (self.integrate(exc) + 0.5 * self.integrate(rho_out, vh_out)
                      - self.integrate(rho_out, veff - self.vloc))
            energy = float(np.sum(2.0 * occ * w)) + e_grid + self.e_nn
            hist_in.append(rho_in)
            hist_out.append(rho_out)
            if len(hist_in) > cfg.history:
                hist_in.pop(0)
                hist_out.pop(0)
            de = None if e_old is None else abs(energy - e_old) / self.natoms
            history.append({"iter": it, "energy": energy, "de_atom": de, "eig": w.copy()})
            e_old = energy
            if de is not None and de < cfg.tol_e_atom:
                break
        return {"history": history, "energy": history[-1]["energy"], "iterations": len(history)}

    def anderson(self, hin, hout):
        from ttdft_public_gb300.scf import solve_small
        h = len(hin)
        F = [hout[i] - hin[i] for i in range(h)]
        n = h - 1
        Fn = F[h - 1]
        D = [Fn - F[h - 2 - mm] for mm in range(n)]
        A = np.array([[self.integrate(D[a], D[b]) for b in range(n)] for a in range(n)])
        b = np.array([self.integrate(D[a], Fn) for a in range(n)])
        c = solve_small(A, b) if n > 0 else np.zeros(0)
        rin = hin[h - 1] + sum(c[kk] * (hin[h - 2 - kk] - hin[h - 1]) for kk in range(n))
        rout = hout[h - 1] + sum(c[kk] * (hout[h - 2 - kk] - hout[h - 1]) for kk in range(n))
        a = self.cfg.mix_alpha
        return np.abs(a * rout + (1.0 - a) * rin)
