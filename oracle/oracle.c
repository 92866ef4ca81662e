/*
 * oracle.c -- FP64 CPU restatement of the reference's ChFSI hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library
 * (libttg.so) is compared against, and the timed CPU baseline of bench.py;
 * it is never linked into, called by or shipped with the product path.
 *
 * Parity status: the reference cannot be built here (PETSc, SLEPc, TuckerMPI,
 * MPI, Boost and ALGLIB are absent, and its only SpMM call, cusparseDcsrmm,
 * was removed after CUDA 10) and it ships no tests or golden vectors, so
 * this restatement is pinned by (a) known-answer tests against numpy/scipy
 * LAPACK and dense formulas in tests/, (b) golden fixtures generated by it
 * and committed under tests/golden/, and (c) mathematical invariants.  Parity
 * to the reference binary itself is unpinned.
 *
 * Layout: dense blocks are column-major N x k (the reference's PETSc dense
 * Mats); CSR uses int64 row pointers and int32 columns.  Functions follow:
 *   or_apply_h        ChebyShevFilter.cc:97-124 (H_loc X + C_nloc_trans (C_nloc X))
 *   or_cheb_filter    ChebyShevFilter.cc:34-189 (incl. the degree m-1 return)
 *   or_lanczos        EigenSolver.cc:186-317 (the T matrix; its eig is in numpy)
 *   or_gram           MultTm.cu:86-224 (X^T Y)
 *   or_cholqr         MultTm.cu:226-467 (S = X^T X = L L^T, X <- X L^-T)
 *   or_rotate         main.cc:1186-1207 (X <- X Q)
 *   or_fermi          KSDFTEnergyFunctional.cc:76-124 + main.cc:1239-1272
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Y = A X for CSR A (rows x cols) and row-major X (cols x k), Y row-major */
static void csr_mm_rows(int64_t rows, const int64_t* rp, const int32_t* col, const double* val,
                        const double* X, int k, double* Y) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < rows; ++i) {
    double* y = Y + i * k;
    for (int c = 0; c < k; ++c) y[c] = 0.0;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
      const double h = val[e];
      const double* x = X + (int64_t)col[e] * k;
      for (int c = 0; c < k; ++c) y[c] += h * x[c];
    }
  }
}

static void to_rows(const double* Xc, int64_t n, int k, double* Xr) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < k; ++c) Xr[i * k + c] = Xc[i + (int64_t)c * n];
}

static void to_cols(const double* Xr, int64_t n, int k, double* Xc) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < k; ++c) Xc[i + (int64_t)c * n] = Xr[i * k + c];
}

/* Yr = H Xr + C^T (D (C Xr)), all row-major; W scratch (nproj x k) */
static void apply_h_rows(int64_t n, const int64_t* hp, const int32_t* hc, const double* hv,
                         int nproj, const int64_t* cp, const int32_t* cc, const double* cv,
                         const double* d, const double* Xr, int k, double* Yr, double* W) {
  csr_mm_rows(n, hp, hc, hv, Xr, k, Yr);
  if (nproj <= 0) return;
  /* C_nloc X = D (C X)   (ProjectHamiltonianSparse.cc:323-325) */
  csr_mm_rows(nproj, cp, cc, cv, Xr, k, W);
  for (int a = 0; a < nproj; ++a)
    for (int c = 0; c < k; ++c) W[(int64_t)a * k + c] *= d[a];
  /* C_nloc_trans (C_nloc X): scatter by projector row (serial over a: few rows) */
  for (int a = 0; a < nproj; ++a)
    for (int64_t e = cp[a]; e < cp[a + 1]; ++e) {
      double* y = Yr + (int64_t)cc[e] * k;
      const double h = cv[e];
      const double* w = W + (int64_t)a * k;
      for (int c = 0; c < k; ++c) y[c] += h * w[c];
    }
}

void or_apply_h(int64_t n, const int64_t* hp, const int32_t* hc, const double* hv, int nproj,
                const int64_t* cp, const int32_t* cc, const double* cv, const double* d,
                const double* X, int k, double* Y) {
  double* Xr = malloc(sizeof(double) * n * k);
  double* Yr = malloc(sizeof(double) * n * k);
  double* W = malloc(sizeof(double) * (nproj > 0 ? nproj : 1) * k);
  to_rows(X, n, k, Xr);
  apply_h_rows(n, hp, hc, hv, nproj, cp, cc, cv, d, Xr, k, Yr, W);
  to_cols(Yr, n, k, Y);
  free(Xr);
  free(Yr);
  free(W);
}

/* Chebyshev filter in place on X (column-major N x k).  Degrees and scalars
 * as ChebyShevFilter.cc:68-75, :129-170.  return_prev = 1 returns the degree
 * m-1 iterate exactly as the reference does (:172-176); 0 returns degree m.
 * steps_limit >= 0 stops after that many operator applications (bounded
 * samples for timing); -1 runs them all. */
void or_cheb_filter(int64_t n, const int64_t* hp, const int32_t* hc, const double* hv, int nproj,
                    const int64_t* cp, const int32_t* cc, const double* cv, const double* d,
                    double* X, int k, int m, double a, double b, double a0, int return_prev,
                    int steps_limit) {
  const double e = (b - a) / 2.0, c = (b + a) / 2.0;
  double sigma = e / (a0 - c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  double alpha = sigma1 / e, beta = alpha * (-c);
  if (m < 1) return;
  double* Xp = malloc(sizeof(double) * n * k);
  double* Yp = malloc(sizeof(double) * n * k);
  double* Yn = malloc(sizeof(double) * n * k);
  double* W = malloc(sizeof(double) * (nproj > 0 ? nproj : 1) * k);
  to_rows(X, n, k, Xp);
  int applied = 0;
  /* Yp = alpha*(H Xp) + beta*Xp */
  apply_h_rows(n, hp, hc, hv, nproj, cp, cc, cv, d, Xp, k, Yp, W);
  applied++;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n * k; ++i) Yp[i] = alpha * Yp[i] + beta * Xp[i];
  for (int deg = 2; deg <= m; ++deg) {
    if (steps_limit >= 0 && applied >= steps_limit) break;
    const double sigma2 = 1.0 / (gamma - sigma);
    alpha = 2.0 * sigma2 / e;
    beta = -c * alpha;
    const double delta = -sigma * sigma2;
    apply_h_rows(n, hp, hc, hv, nproj, cp, cc, cv, d, Yp, k, Yn, W);
    applied++;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n * k; ++i) Yn[i] = alpha * Yn[i] + beta * Yp[i] + delta * Xp[i];
    double* t = Xp;
    Xp = Yp;
    Yp = Yn;
    Yn = t;
    sigma = sigma2;
  }
  to_cols(return_prev ? Xp : Yp, n, k, X);
  free(Xp);
  free(Yp);
  free(Yn);
  free(W);
}

/* Lanczos (EigenSolver.cc:195-317) from a given start vector v (length n).
 * Outputs alpha[0..it-1], beta[0..it-1]; beta[it-1] is the final |f|. */
void or_lanczos(int64_t n, const int64_t* hp, const int32_t* hc, const double* hv, int nproj,
                const int64_t* cp, const int32_t* cc, const double* cv, const double* d,
                const double* v_in, int maxit, double* alpha, double* beta) {
  double* v = malloc(sizeof(double) * n);
  double* v0 = malloc(sizeof(double) * n);
  double* f = malloc(sizeof(double) * n);
  double* W = malloc(sizeof(double) * (nproj > 0 ? nproj : 1));
  double nv = 0.0;
  for (int64_t i = 0; i < n; ++i) nv += v_in[i] * v_in[i];
  nv = sqrt(nv);
  for (int64_t i = 0; i < n; ++i) v[i] = v_in[i] / nv;
  apply_h_rows(n, hp, hc, hv, nproj, cp, cc, cv, d, v, 1, f, W);
  double al = 0.0;
  for (int64_t i = 0; i < n; ++i) al += f[i] * v[i];
  for (int64_t i = 0; i < n; ++i) f[i] -= al * v[i];
  alpha[0] = al;
  for (int it = 1; it < maxit; ++it) {
    double be = 0.0;
    for (int64_t i = 0; i < n; ++i) be += f[i] * f[i];
    be = sqrt(be);
    beta[it - 1] = be;
    for (int64_t i = 0; i < n; ++i) {
      v0[i] = v[i];
      v[i] = f[i] / be;
    }
    apply_h_rows(n, hp, hc, hv, nproj, cp, cc, cv, d, v, 1, f, W);
    for (int64_t i = 0; i < n; ++i) f[i] -= be * v0[i];
    al = 0.0;
    for (int64_t i = 0; i < n; ++i) al += v[i] * f[i];
    for (int64_t i = 0; i < n; ++i) f[i] -= al * v[i];
    alpha[it] = al;
  }
  double be = 0.0;
  for (int64_t i = 0; i < n; ++i) be += f[i] * f[i];
  beta[maxit - 1] = sqrt(be);
  free(v);
  free(v0);
  free(f);
  free(W);
}

/* S = X^T Y, X, Y column-major N x k, S column-major k x k */
void or_gram(int64_t n, int k, const double* X, const double* Y, double* S) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int p = 0; p < k; ++p)
    for (int q = 0; q < k; ++q) {
      const double* x = X + (int64_t)p * n;
      const double* y = Y + (int64_t)q * n;
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
      S[p + (int64_t)q * k] = s;
    }
}

/* Cholesky-QR: returns 0, or j+1 when pivot j is not positive relative to
 * the diagonal entry it started from (pivot <= 1e-12 * S_jj: the columns are
 * numerically dependent and X L^-T would not be orthonormal in FP64). */
int or_cholqr(int64_t n, int k, double* X) {
  double* S = malloc(sizeof(double) * k * k);
  or_gram(n, k, X, X, S);
  /* lower Cholesky in place (column-major) */
  for (int j = 0; j < k; ++j) {
    const double s0 = S[j + (int64_t)j * k];
    double dj = s0;
    for (int p = 0; p < j; ++p) dj -= S[j + (int64_t)p * k] * S[j + (int64_t)p * k];
    if (!(dj > 1e-12 * s0) || !(s0 > 0.0)) {
      free(S);
      return j + 1;
    }
    dj = sqrt(dj);
    S[j + (int64_t)j * k] = dj;
    for (int i = j + 1; i < k; ++i) {
      double s = S[i + (int64_t)j * k];
      for (int p = 0; p < j; ++p) s -= S[i + (int64_t)p * k] * S[j + (int64_t)p * k];
      S[i + (int64_t)j * k] = s / dj;
    }
  }
  /* X <- X L^-T: each row x solves z L^T = x, i.e. L z^T = x^T (forward) */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double z[4096];
    for (int j = 0; j < k; ++j) {
      double s = X[i + (int64_t)j * n];
      for (int p = 0; p < j; ++p) s -= S[j + (int64_t)p * k] * z[p];
      z[j] = s / S[j + (int64_t)j * k];
    }
    for (int j = 0; j < k; ++j) X[i + (int64_t)j * n] = z[j];
  }
  free(S);
  return 0;
}

/* X <- X Q, Q column-major k x k */
void or_rotate(int64_t n, int k, double* X, const double* Q) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double row[4096];
    for (int p = 0; p < k; ++p) row[p] = X[i + (int64_t)p * n];
    for (int q = 0; q < k; ++q) {
      double s = 0.0;
      for (int p = 0; p < k; ++p) s += row[p] * Q[p + (int64_t)q * k];
      X[i + (int64_t)q * n] = s;
    }
  }
}

/* Fermi level by Newton and occupancies; returns iterations used */
int or_fermi(const double* eig, int k, int n_electrons, double kT, int max_iter, double* mu_out,
             double* occ) {
  int occ_num = n_electrons / 2;
  if (n_electrons % 2 == 1) occ_num += 1;
  double mu = eig[occ_num - 1];
  int it = 0;
  for (; it < max_iter; ++it) {
    double sf = 0.0, sd = 0.0;
    for (int i = 0; i < k; ++i) {
      const double arg = (eig[i] - mu) / kT;
      if (arg <= 0.0) {
        const double t = 1.0 / (1.0 + exp(arg));
        sf += 2.0 * t;
        sd += 2.0 * (exp(arg) / kT) * t * t;
      } else {
        const double t = 1.0 / (1.0 + exp(-arg));
        sf += 2.0 * exp(-arg) * t;
        sd += 2.0 * (exp(-arg) / kT) * t * t;
      }
    }
    const double func = sf - n_electrons;
    mu -= func / sd;
    if (fabs(func) <= 1.0e-8) break;
  }
  for (int i = 0; i < k; ++i) {
    const double term = (eig[i] - mu) / kT;
    occ[i] = term <= 0.0 ? 1.0 / (1.0 + exp(term)) : exp(-term) / (1.0 + exp(-term));
  }
  *mu_out = mu;
  return it;
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
