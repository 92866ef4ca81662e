// FP64 dense kernels of the Rayleigh-Ritz step.
//
//   gram_tn        S = X^T Y (k x k), split over rows with a fixed-order
//                  reduction of the partial tiles (bitwise reproducible).
//                  MultTM::mult, eigensolver/MultTm.cu:86-224.
//   gemm_nn_small  out = X Q or X Q^T, Q k x k.  Subspace rotation
//                  (main.cc:1186-1207) and the X L^-T of Cholesky-QR
//                  (eigensolver/MultTm.cu:422-438 / the SOLVE_WITH_INVERSE
//                  variant :309-404).
//   cholesky_inv   S = L L^T and L^-1, status on a non-positive pivot
//                  (the reference ignores potrf's info, MultTm.cu:283-294).
//   syev_device    symmetric eigensolver: Householder tridiagonalisation +
//                  implicit QL in FP32, then FP64 iterative refinement
//                  (Ogita-Aishima); ascending eigenvalues.  Replaces the
//                  SLEPc/LAPACK call of EigenSolver::computeEigenPairsSeq
//                  (EigenSolver.cc:30-184).
//   lanczos_step   one Lanczos three-term step on the device
//                  (EigenSolver.cc:262-315).
//   fermi          Newton iteration for the Fermi level
//                  (dft/KSDFTEnergyFunctional.cc:76-124) and occupations
//                  (main.cc:1239-1272).
//
// FP64 throughout: these are the quantities the method keeps in double.  The
// two N x k GEMMs (the Gram X^T Y and the rotation X Q) read and write FP64
// and compute in double-FP32 on the FP32 pipe (about 48 bits; FP64 runs at
// a small fraction of the FP32 rate on this part).

#include <algorithm>
#include <cmath>
#include <mutex>
#include "ttg_internal.cuh"

namespace ttg {
namespace {

constexpr int TM = 64, TN = 64, TK = 16;

// S_partial[z] = X[rows_z]^T Y[rows_z]; 256 threads, 4x4 outputs each.
// sym: blockIdx.x enumerates the tiles on and below the diagonal (tile row
// pt >= tile column qt, row-major over the triangle), blockIdx.y is 0; the
// other tiles are not computed (k_reduce_splits mirrors them).
__global__ void __launch_bounds__(256) k_gram_tn(const double* __restrict__ X,
                                                 const double* __restrict__ Y, int64_t n,
                                                 int k, int64_t ld, int64_t rows_per_split,
                                                 double* __restrict__ part, int sym) {
  __shared__ float sXh[TK][TM + 1], sXl[TK][TM + 1];
  __shared__ float sYh[TK][TN + 1], sYl[TK][TN + 1];
  int pt = blockIdx.x, qt = blockIdx.y;
  if (sym) {
    const int t = blockIdx.x;
    pt = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while (pt * (pt + 1) / 2 > t) --pt;
    while ((pt + 1) * (pt + 2) / 2 <= t) ++pt;
    qt = t - pt * (pt + 1) / 2;
  }
  const int p0 = pt * TM, q0 = qt * TN;
  const int64_t r0 = (int64_t)blockIdx.z * rows_per_split;
  const int64_t r1 = (n < r0 + rows_per_split ? n : r0 + rows_per_split);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  F2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = F2{0.f, 0.f};
  for (int64_t rb = r0; rb < r1; rb += TK) {
    for (int i = threadIdx.x; i < TK * TM; i += 256) {
      const int rr = i / TM, cc = i % TM;
      const int64_t row = rb + rr;
      const F2 xv = to_f2((row < r1 && p0 + cc < k) ? X[row * ld + p0 + cc] : 0.0);
      const F2 yv = to_f2((row < r1 && q0 + cc < k) ? Y[row * ld + q0 + cc] : 0.0);
      sXh[rr][cc] = xv.h;
      sXl[rr][cc] = xv.l;
      sYh[rr][cc] = yv.h;
      sYl[rr][cc] = yv.l;
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < TK; ++t) {
      F2 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = F2{sXh[t][ty + 16 * u], sXl[t][ty + 16 * u]};
        b[u] = F2{sYh[t][tx + 16 * u], sYl[t][tx + 16 * u]};
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) f2_fma(acc[u][v], a[u], b[v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) f2_renorm(acc[u][v]);
    __syncthreads();
  }
  double* out = part + (int64_t)blockIdx.z * k * k;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int p = p0 + ty + 16 * u, q = q0 + tx + 16 * v;
      if (p < k && q < k)     // column-major
        out[p + (int64_t)q * k] = (double)acc[u][v].h + (double)acc[u][v].l;
    }
}

// S = sum of the split partials.  sym (k > 0): only tiles with tile row >=
// tile column were computed; S[p, q] for a tile above the diagonal is read
// from its mirror [q, p].
__global__ void k_reduce_splits(const double* __restrict__ part, int nsplit, int64_t kk,
                                double* __restrict__ S, int sym_k) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kk;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t src = i;
    if (sym_k > 0) {
      const int p = (int)(i % sym_k), q = (int)(i / sym_k);
      if (p / TM < q / TN) src = q + (int64_t)p * sym_k;
    }
    double s = 0.0;
    for (int z = 0; z < nsplit; ++z) s += part[(int64_t)z * kk + src];
    S[i] = s;
  }
}

// out[i, q] = sum_p X[i, p] * Qop[p, q],  Qop = Q or Q^T (Q column-major k x k).
// transQ with Q lower triangular (L^-1): Qop[p, q] = 0 for p > q, so the sum
// for the tile's columns [q0, q0 + TN) stops at q0 + TN.
__global__ void __launch_bounds__(256) k_gemm_nn(const double* __restrict__ X,
                                                 const double* __restrict__ Q,
                                                 double* __restrict__ out, int64_t n, int k,
                                                 int64_t ld, int transQ, int lower) {
  __shared__ float sXh[TM][TK + 1], sXl[TM][TK + 1];
  __shared__ float sQh[TK][TN + 1], sQl[TK][TN + 1];
  const int64_t i0 = (int64_t)blockIdx.x * TM;
  const int q0 = blockIdx.y * TN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  F2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = F2{0.f, 0.f};
  const int kend = (transQ && lower) ? min(k, q0 + TN) : k;
  for (int pb = 0; pb < kend; pb += TK) {
    for (int e = threadIdx.x; e < TM * TK; e += 256) {
      const int rr = e / TK, cc = e % TK;
      const int64_t row = i0 + rr;
      const F2 xv = to_f2((row < n && pb + cc < k) ? X[row * ld + pb + cc] : 0.0);
      sXh[rr][cc] = xv.h;
      sXl[rr][cc] = xv.l;
    }
    for (int e = threadIdx.x; e < TK * TN; e += 256) {
      const int rr = e / TN, cc = e % TN;
      const int p = pb + rr, q = q0 + cc;
      double v = 0.0;
      if (p < k && q < k) v = transQ ? Q[q + (int64_t)p * k] : Q[p + (int64_t)q * k];
      const F2 qv = to_f2(v);
      sQh[rr][cc] = qv.h;
      sQl[rr][cc] = qv.l;
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < TK; ++t) {
      F2 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = F2{sXh[ty + 16 * u][t], sXl[ty + 16 * u][t]};
        b[u] = F2{sQh[t][tx + 16 * u], sQl[t][tx + 16 * u]};
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) f2_fma(acc[u][v], a[u], b[v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) f2_renorm(acc[u][v]);
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int64_t i = i0 + ty + 16 * u;
      const int q = q0 + tx + 16 * v;
      if (i < n && q < k) out[i * ld + q] = (double)acc[u][v].h + (double)acc[u][v].l;
    }
}

template <typename T>
__device__ T block_sum(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  T s = T(0);
  const int nw = (blockDim.x + 31) / 32;
  for (int i = 0; i < nw; ++i) s += red[i];
  return s;
}

// Right-looking Cholesky in place on the lower triangle of A (column-major),
// then Linv = L^-1 (lower).  One CTA.  status[0] = 0 ok, j+1 if pivot j <= 0.
__global__ void __launch_bounds__(1024) k_cholesky_inv(double* A, double* Linv, int k,
                                                       int* status) {
  __shared__ double s_piv;
  __shared__ int s_bad;
  // diagonal of S before the factorisation, for the relative pivot test
  double* diag0 = Linv;
  for (int j = threadIdx.x; j < k; j += blockDim.x) diag0[j] = A[j + (int64_t)j * k];
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    if (threadIdx.x == 0) {
      const double d = A[j + (int64_t)j * k];
      const double s0 = diag0[j];
      // not positive definite in FP64: pivot lost 12+ digits of its diagonal
      if (!(d > 1e-12 * s0) || !(s0 > 0.0) || !isfinite(d)) s_bad = j + 1;
      s_piv = d > 0.0 ? sqrt(d) : 1.0;
    }
    __syncthreads();
    if (s_bad) break;
    const double piv = s_piv;
    for (int i = j + threadIdx.x; i < k; i += blockDim.x) {
      const double v = (i == j) ? piv : A[i + (int64_t)j * k] / piv;
      A[i + (int64_t)j * k] = v;
    }
    __syncthreads();
    // trailing update of the lower triangle: A[i,l] -= L[i,j] L[l,j], j<l<=i
    const int m = k - j - 1;
    for (int64_t e = threadIdx.x; e < (int64_t)m * m; e += blockDim.x) {
      const int ii = (int)(e % m), ll = (int)(e / m);
      if (ll > ii) continue;
      const int i = j + 1 + ii, l = j + 1 + ll;
      A[i + (int64_t)l * k] -= A[i + (int64_t)j * k] * A[l + (int64_t)j * k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) status[0] = s_bad;
  if (s_bad) return;
  // Linv: row by row, X[i][j] = (delta_ij - sum_{p=j}^{i-1} L[i,p] X[p][j]) / L[i,i]
  __syncthreads();
  for (int64_t e = threadIdx.x; e < (int64_t)k * k; e += blockDim.x) Linv[e] = 0.0;
  __syncthreads();
  for (int i = 0; i < k; ++i) {
    const double lii = A[i + (int64_t)i * k];
    for (int j = threadIdx.x; j <= i; j += blockDim.x) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int p = j; p < i; ++p) s -= A[i + (int64_t)p * k] * Linv[p + (int64_t)j * k];
      Linv[i + (int64_t)j * k] = s / lii;
    }
    __syncthreads();
  }
}

// Symmetric eigensolver in two stages, one CTA (run in FP32 here):
//  (1) Householder reduction to tridiagonal form, A = Q T Q^T: for each
//      column j, v = x - alpha e1 with x = A[j+1:, j], P = I - tau v v^T and
//      the trailing block is updated as B <- P B P = B - v w^T - w v^T with
//      p = tau B v, w = p - (tau/2)(v.p) v; Q accumulates the reflectors.
//  (2) implicit QL iterations with Wilkinson-type shifts on T (the classical
//      tql algorithm), one thread running the scalar recurrence and storing
//      each sweep's plane rotations, all threads then applying them to their
//      own rows of Q.
// 4n^3/3 flops for (1) plus O(n^2) rotations on Q in (2), against ~10
// sweeps of 3n^3 for Jacobi.  The vectors, the tridiagonal and the rotations
// live in shared memory (6n elements, dynamic): the QL recurrence is a serial
// chain of dependent accesses.  status[0]: 0 ok, 1 QL did not converge.
template <typename T>
__global__ void __launch_bounds__(1024) k_tridiag_ql(T* A, T* Q, T* w, int n, int* status,
                                                     T* scratch) {
  const T kTiny = sizeof(T) == 4 ? T(1.2e-7) : T(1e-16);
  __shared__ T red[32];
  __shared__ T s_alpha, s_tau;
  extern __shared__ __align__(16) unsigned char ql_smem[];
  T* v = reinterpret_cast<T*>(ql_smem);   // n
  T* p = v + n;                 // n
  T* d = p + n;                 // n
  T* e = d + n;                 // n
  T* rot = e + n;               // 2n: (c, s) of one QL sweep
  T* vs = scratch;              // n*n: reflectors, column j holds v_j (rows j+1..)
  const int tid = threadIdx.x, nt = blockDim.x;
  // ---- (1) tridiagonalisation
  for (int j = 0; j + 2 < n; ++j) {
    const int m = n - j - 1;
    T ss = 0.0;
    for (int r = tid; r < m; r += nt) {
      const T x = A[(j + 1 + r) + (int64_t)j * n];
      ss += x * x;
    }
    ss = block_sum(ss, red);
    if (tid == 0) {
      const T x0 = A[(j + 1) + (int64_t)j * n];
      const T nrm = sqrt(ss);
      const T alpha = x0 >= 0 ? -nrm : nrm;
      const T vnorm2 = ss - x0 * x0 + (x0 - alpha) * (x0 - alpha);
      s_alpha = alpha;
      s_tau = vnorm2 > T(0) ? T(2) / vnorm2 : T(0);
    }
    __syncthreads();
    const T alpha = s_alpha, tau = s_tau;
    for (int r = tid; r < m; r += nt) {
      const T x = A[(j + 1 + r) + (int64_t)j * n];
      const T vr = (r == 0) ? x - alpha : x;
      v[r] = vr;
      vs[(j + 1 + r) + (int64_t)j * n] = vr;
    }
    __syncthreads();
    if (tau == T(0)) continue;
    // p = tau B v  (B = A[j+1:, j+1:], column-major)
    for (int r = tid; r < m; r += nt) {
      T acc = 0.0;
      for (int c = 0; c < m; ++c) acc += A[(j + 1 + r) + (int64_t)(j + 1 + c) * n] * v[c];
      p[r] = tau * acc;
    }
    __syncthreads();
    T vp = 0.0;
    for (int r = tid; r < m; r += nt) vp += v[r] * p[r];
    vp = block_sum(vp, red);
    const T K = T(0.5) * tau * vp;
    for (int r = tid; r < m; r += nt) p[r] -= K * v[r];   // p becomes w
    __syncthreads();
    for (int64_t e2 = tid; e2 < (int64_t)m * m; e2 += nt) {
      const int r = (int)(e2 % m), c = (int)(e2 / m);
      A[(j + 1 + r) + (int64_t)(j + 1 + c) * n] -= v[r] * p[c] + p[r] * v[c];
    }
    if (tid == 0) {
      A[(j + 1) + (int64_t)j * n] = alpha;
      A[j + (int64_t)(j + 1) * n] = alpha;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += nt) {
    d[i] = A[i + (int64_t)i * n];
    e[i] = (i + 1 < n) ? A[(i + 1) + (int64_t)i * n] : 0.0;
  }
  // Q = P_0 P_1 ... P_{n-3}, built backwards: Q <- P_j Q on rows/cols j+1..
  for (int64_t e2 = tid; e2 < (int64_t)n * n; e2 += nt) {
    const int r = (int)(e2 % n), c = (int)(e2 / n);
    Q[e2] = (r == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int j = n - 3; j >= 0; --j) {
    const int m = n - j - 1;
    T vn = 0.0;
    for (int r = tid; r < m; r += nt) {
      const T x = vs[(j + 1 + r) + (int64_t)j * n];
      vn += x * x;
    }
    vn = block_sum(vn, red);
    if (vn == T(0)) continue;
    const T tau = T(2) / vn;
    // columns c of the trailing block: Q[:, c] -= tau v (v . Q[:, c])
    for (int c = tid; c < m; c += nt) {
      T dot = 0.0;
      for (int r = 0; r < m; ++r)
        dot += vs[(j + 1 + r) + (int64_t)j * n] * Q[(j + 1 + r) + (int64_t)(j + 1 + c) * n];
      p[c] = tau * dot;
    }
    __syncthreads();
    for (int64_t e2 = tid; e2 < (int64_t)m * m; e2 += nt) {
      const int r = (int)(e2 % m), c = (int)(e2 / m);
      Q[(j + 1 + r) + (int64_t)(j + 1 + c) * n] -= vs[(j + 1 + r) + (int64_t)j * n] * p[c];
    }
    __syncthreads();
  }
  // ---- (2) implicit QL on (d, e), rotations applied to the rows of Q
  __shared__ int s_m, s_done, s_fail, s_nrot;
  __shared__ T s_floor;
  if (tid == 0) {
    s_fail = 0;
    T tn = T(0);
    for (int i = 0; i < n; ++i) tn = fmax(tn, fabs(d[i]) + fabs(e[i]));
    // off-diagonals below kTiny^2 |T| are zero at this precision
    s_floor = kTiny * kTiny * tn;
  }
  __syncthreads();
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      if (tid == 0) {
        int m = l;
        for (; m < n - 1; ++m) {
          const T dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= kTiny * dd || fabs(e[m]) <= s_floor) break;
        }
        s_m = m;
        s_done = (m == l);
        s_nrot = 0;
        if (!s_done) {
          if (++iter > 100) {
            s_fail = 1;
            s_done = 1;
          } else {
            T g = (d[l + 1] - d[l]) / (T(2) * e[l]);
            T r = hypot(g, T(1));
            g = d[m] - d[l] + e[l] / (g + (g >= 0 ? fabs(r) : -fabs(r)));
            T s = T(1), c = T(1), pp = T(0);
            int i = m - 1;
            bool underflow = false;
            for (; i >= l; --i) {
              const T f = s * e[i], b = c * e[i];
              r = hypot(f, g);
              e[i + 1] = r;
              if (r == T(0)) {
                d[i + 1] -= pp;
                e[m] = T(0);
                underflow = true;
                break;
              }
              s = f / r;
              c = g / r;
              g = d[i + 1] - pp;
              r = (d[i] - g) * s + T(2) * c * b;
              pp = s * r;
              d[i + 1] = g + pp;
              g = c * r - b;
              rot[2 * s_nrot] = c;
              rot[2 * s_nrot + 1] = s;
              s_nrot++;
            }
            if (!underflow) {
              d[l] -= pp;
              e[l] = g;
              e[m] = T(0);
            }
          }
        }
      }
      __syncthreads();
      if (s_done) break;
      // rotation q (i = m-1-q) mixes columns i and i+1 of Q, for every row
      const int m = s_m, nr = s_nrot;
      for (int row = tid; row < n; row += nt) {
        for (int q = 0; q < nr; ++q) {
          const int i = m - 1 - q;
          const T c = rot[2 * q], s = rot[2 * q + 1];
          const T f = Q[row + (int64_t)(i + 1) * n];
          const T zi = Q[row + (int64_t)i * n];
          Q[row + (int64_t)(i + 1) * n] = s * zi + c * f;
          Q[row + (int64_t)i * n] = c * zi - s * f;
        }
      }
      __syncthreads();
    }
    if (s_fail) break;
  }
  for (int i = tid; i < n; i += nt) w[i] = d[i];
  if (tid == 0) status[0] = s_fail;
}

// Sort eigenpairs ascending (stable rank sort), normalise each eigenvector's
// sign so that its largest-magnitude component is positive.
__global__ void k_sort_eig(const double* w, const double* V, double* w_out, double* V_out,
                           int k) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < k; j += gridDim.x * blockDim.x) {
    int rank = 0;
    const double wj = w[j];
    for (int i = 0; i < k; ++i) rank += (w[i] < wj) || (w[i] == wj && i < j);
    w_out[rank] = wj;
    double big = 0.0;
    int ib = 0;
    for (int i = 0; i < k; ++i) {
      const double a = fabs(V[i + (int64_t)j * k]);
      if (a > big) { big = a; ib = i; }
    }
    const double sg = V[ib + (int64_t)j * k] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < k; ++i) V_out[i + (int64_t)rank * k] = sg * V[i + (int64_t)j * k];
  }
}

// One step of the Ogita-Aishima iterative refinement of a symmetric
// eigendecomposition (Ogita & Aishima, Japan J. Indust. Appl. Math. 35 (2018)):
// with G = V^T V, S = V^T A V, r_ij = delta_ij - G_ij, lam_i = S_ii / G_ii,
// delta = 2 (|S - diag(lam)| + |A| |R|) (Frobenius norms, bounds of the 2-norms),
// E_ij = (S_ij + lam_j r_ij) / (lam_j - lam_i) if |lam_i - lam_j| > delta, else r_ij / 2;
// the caller then forms V <- V + V E.  One CTA.
__global__ void __launch_bounds__(1024) k_oa_step(const double* __restrict__ G,
                                                  const double* __restrict__ S, int k,
                                                  const double* __restrict__ normA, double* E,
                                                  double* lam) {
  __shared__ double red[32];
  for (int i = threadIdx.x; i < k; i += blockDim.x) lam[i] = S[i + (int64_t)i * k] / G[i + (int64_t)i * k];
  __syncthreads();
  double sd = 0.0, rr = 0.0;
  for (int64_t e = threadIdx.x; e < (int64_t)k * k; e += blockDim.x) {
    const int i = (int)(e % k), j = (int)(e / k);
    const double sij = S[e] - (i == j ? lam[i] : 0.0);
    const double rij = (i == j ? 1.0 : 0.0) - G[e];
    sd += sij * sij;
    rr += rij * rij;
  }
  sd = block_sum(sd, red);
  rr = block_sum(rr, red);
  const double delta = 2.0 * (sqrt(sd) + sqrt(*normA) * sqrt(rr));
  for (int64_t e = threadIdx.x; e < (int64_t)k * k; e += blockDim.x) {
    const int i = (int)(e % k), j = (int)(e / k);
    const double rij = (i == j ? 1.0 : 0.0) - G[e];
    const double gap = lam[j] - lam[i];
    E[e] = fabs(gap) > delta ? (S[e] + lam[j] * rij) / gap : 0.5 * rij;
  }
}

__global__ void k_frob2(const double* __restrict__ A, int64_t n, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) s += A[e] * A[e];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_add(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    a[e] += b[e];
}

__global__ void k_d2f_vec(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    b[e] = (float)a[e];
}

__global__ void k_f2d_vec(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    b[e] = (double)a[e];
}

__global__ void k_symmetrize(double* A, int k) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)k * k;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % k), j = (int)(e / k);
    if (i < j) {
      const double v = 0.5 * (A[i + (int64_t)j * k] + A[j + (int64_t)i * k]);
      A[i + (int64_t)j * k] = v;
      A[j + (int64_t)i * k] = v;
    }
  }
}

__global__ void k_cm_to_rows(const double* __restrict__ src, int64_t lds, double* __restrict__ dst,
                             int64_t ldd, int64_t n, int k) {
  // tile transpose 32x32
  __shared__ double t[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32;
  const int j0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int j = j0 + y;
    const int64_t i = i0 + threadIdx.x;
    t[y][threadIdx.x] = (i < n && j < k) ? src[i + (int64_t)j * lds] : 0.0;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t i = i0 + y;
    const int j = j0 + threadIdx.x;
    if (i < n && j < k) dst[i * ldd + j] = t[threadIdx.x][y];
  }
}

__global__ void k_rows_to_cm(const double* __restrict__ src, int64_t lds, double* __restrict__ dst,
                             int64_t ldd, int64_t n, int k) {
  __shared__ double t[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32;
  const int j0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t i = i0 + y;
    const int j = j0 + threadIdx.x;
    t[y][threadIdx.x] = (i < n && j < k) ? src[i * lds + j] : 0.0;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int j = j0 + y;
    const int64_t i = i0 + threadIdx.x;
    if (i < n && j < k) dst[i + (int64_t)j * ldd] = t[threadIdx.x][y];
  }
}

// One Lanczos step on strided vectors (stride ld).  Single CTA.
//   f = hv - beta_prev v0;  alpha = v.f;  f -= alpha v;  beta = |f|;
//   v0 <- v;  v <- f / beta;  ab[2*it] = alpha, ab[2*it+1] = beta.
__global__ void __launch_bounds__(1024) k_lanczos_step(double* v, double* v0, const double* hv,
                                                       int64_t n, int64_t ld, double* ab,
                                                       int it) {
  __shared__ double red[32];
  const double beta_prev = it > 0 ? ab[2 * (it - 1) + 1] : 0.0;
  double d = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double f = hv[i * ld] - beta_prev * v0[i * ld];
    d += v[i * ld] * f;
  }
  const double alpha = block_sum(d, red);
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double f = hv[i * ld] - beta_prev * v0[i * ld] - alpha * v[i * ld];
    s += f * f;
  }
  const double beta = sqrt(block_sum(s, red));
  const double inv = beta > 0 ? 1.0 / beta : 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double f = hv[i * ld] - beta_prev * v0[i * ld] - alpha * v[i * ld];
    const double vi = v[i * ld];
    v0[i * ld] = vi;
    v[i * ld] = f * inv;
  }
  if (threadIdx.x == 0) {
    ab[2 * it] = alpha;
    ab[2 * it + 1] = beta;
  }
}

__global__ void __launch_bounds__(1024) k_normalize(double* v, int64_t n, int64_t ld) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i * ld] * v[i * ld];
  const double nrm = sqrt(block_sum(s, red));
  const double inv = nrm > 0 ? 1.0 / nrm : 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) v[i * ld] *= inv;
}

// Fermi level by Newton (dft/KSDFTEnergyFunctional.cc:76-124) and occupancy
// factors (main.cc:1247-1260).  One CTA.  out[0] = mu, out[1] = iterations,
// out[2] = final |sum - Ne|.
__global__ void __launch_bounds__(256) k_fermi(const double* eig, int k, double ne, double kT,
                                               int max_iter, double* occ, double* out) {
  __shared__ double red[32];
  int occ_num = (int)(ne / 2.0);
  if (((long long)ne) % 2 == 1) occ_num += 1;
  occ_num = max(1, min(occ_num, k));
  double mu = eig[occ_num - 1];
  int it = 0;
  double func = 0.0;
  for (; it < max_iter; ++it) {
    double sf = 0.0, sd = 0.0;
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
      const double arg = (eig[i] - mu) / kT;
      if (arg <= 0.0) {
        const double term = 1.0 / (1.0 + exp(arg));
        sf += 2.0 * term;
        sd += 2.0 * (exp(arg) / kT) * term * term;
      } else {
        const double term = 1.0 / (1.0 + exp(-arg));
        sf += 2.0 * exp(-arg) * term;
        sd += 2.0 * (exp(-arg) / kT) * term * term;
      }
    }
    sf = block_sum(sf, red);
    sd = block_sum(sd, red);
    func = sf - ne;
    mu = mu - func / sd;
    if (fabs(func) <= 1.0e-8) break;
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const double term = (eig[i] - mu) / kT;
    occ[i] = term <= 0.0 ? 1.0 / (1.0 + exp(term)) : exp(-term) / (1.0 + exp(-term));
  }
  if (threadIdx.x == 0) {
    out[0] = mu;
    out[1] = (double)it;
    out[2] = fabs(func);
  }
}

}  // namespace

ttg_status gram_tn(ttg_op* op, const double* X, const double* Y, int k, double* S, bool sym) {
  const int tp = (k + TM - 1) / TM, tq = (k + TN - 1) / TN;
  const int tiles = sym ? tp * (tp + 1) / 2 : tp * tq;
  int64_t nsplit = (2 * 152 + tiles - 1) / tiles;
  nsplit = std::min<int64_t>(nsplit, (op->n + 255) / 256);
  if (nsplit < 1) nsplit = 1;
  const int64_t need = nsplit * (int64_t)k * k * sizeof(double);
  if ((int64_t)op->partial.bytes < need) TTG_TRY(op->partial.alloc(need));
  const int64_t rows = (op->n + nsplit - 1) / nsplit;
  const dim3 grid = sym ? dim3((unsigned)tiles, 1, (unsigned)nsplit)
                        : dim3((unsigned)tp, (unsigned)tq, (unsigned)nsplit);
  k_gram_tn<<<grid, 256, 0, op->stream>>>(X, Y, op->n, k, op->ld, rows, op->partial.as<double>(),
                                          sym ? 1 : 0); TTG_COUNT();
  TTG_LAUNCHED(op);
  const int64_t kk = (int64_t)k * k;
  k_reduce_splits<<<(unsigned)std::min<int64_t>((kk + 255) / 256, 1024), 256, 0, op->stream>>>(
      op->partial.as<double>(), (int)nsplit, kk, S, sym ? k : 0); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status gemm_nn_small(ttg_op* op, const double* X, const double* Q, double* out, int k,
                         int transQ, bool lower) {
  dim3 grid((unsigned)((op->n + TM - 1) / TM), (unsigned)((k + TN - 1) / TN));
  k_gemm_nn<<<grid, 256, 0, op->stream>>>(X, Q, out, op->n, k, op->ld, transQ,
                                          lower ? 1 : 0); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

// d[i] = sqrt(S_ii) (1 where that is not a positive finite number, counted
// in *bad)
__global__ void k_diag_sqrt(const double* __restrict__ S, int k, double* __restrict__ d,
                            int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) {
    const double v = S[i + (int64_t)i * k];
    const bool ok = v > 0.0 && isfinite(v);
    d[i] = ok ? sqrt(v) : 1.0;
    if (!ok) atomicAdd(bad, 1);
  }
}

// S <- D^-1 S D^-1 + shift I (column-major k x k)
__global__ void k_unit_scale_shift(double* __restrict__ S, const double* __restrict__ d, int k,
                                   double shift) {
  const int64_t n = (int64_t)k * k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % k), j = (int)(e / k);
    S[e] = S[e] / (d[i] * d[j]) + (i == j ? shift : 0.0);
  }
}

// L[:, j] <- L[:, j] / d[j]
__global__ void k_scale_cols(double* __restrict__ L, const double* __restrict__ d, int k) {
  const int64_t n = (int64_t)k * k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    L[e] /= d[e / k];
}

ttg_status unit_scale_shift(ttg_op* op, double* S, double* d, int k, double shift, int* bad) {
  TTG_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), op->stream));
  k_diag_sqrt<<<(k + 255) / 256, 256, 0, op->stream>>>(S, k, d, bad); TTG_COUNT();
  TTG_LAUNCHED(op);
  const unsigned g = (unsigned)std::min<int64_t>(((int64_t)k * k + 255) / 256, 4096);
  k_unit_scale_shift<<<g, 256, 0, op->stream>>>(S, d, k, shift); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status scale_cols(ttg_op* op, double* L, const double* d, int k) {
  const unsigned g = (unsigned)std::min<int64_t>(((int64_t)k * k + 255) / 256, 4096);
  k_scale_cols<<<g, 256, 0, op->stream>>>(L, d, k); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

// ---- blocked Cholesky and inverse (k > kCholSmall), FP64 on many CTAs ----
// A (k x k, column-major, lower triangle used) is factored in place in
// panels of CB columns: the diagonal block in one CTA's shared memory
// (k_chol_diag, which also inverts it into Linv's diagonal block), the panel
// below as A21 inv(L11)^T (k_chol_panel), the trailing lower triangle
// updated by A22 -= L21 L21^T (k_chol_update).  Linv's blocks below the
// diagonal then follow by block forward substitution, one CTA per block
// column and 16-column slice (k_chol_inv_offdiag).  The same relative pivot
// test as k_cholesky_inv: status[0] = j + 1 when pivot j has lost 12 digits
// of its original diagonal.
constexpr int CB = 64;
constexpr int CBP = CB + 1;                  // padded row of a shared tile
constexpr int kCholSmall = 128;
constexpr size_t kTileBytes = (size_t)CB * CBP * sizeof(double);   // 33,280

__global__ void __launch_bounds__(256) k_chol_diag(double* __restrict__ A, int k, int j0, int b,
                                                   const double* __restrict__ diag0,
                                                   double* __restrict__ Linv,
                                                   int* __restrict__ status) {
  // T: the block; its strict upper triangle then holds inv(L11) transposed
  // (V[i][j] at T[j][i], i > j), the diagonal of inv(L11) in Vd
  extern __shared__ double sm[];
  double* T = sm;
  __shared__ double Vd[CB];
  __shared__ int bad;
  if (status[0] != 0) return;
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int i = e % b, j = e / b;
    T[i * CBP + j] = i >= j ? A[(j0 + i) + (int64_t)(j0 + j) * k] : 0.0;
  }
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < b; ++j) {
    if (threadIdx.x == 0) {
      const double d = T[j * CBP + j], s0 = diag0[j0 + j];
      if (!(d > 1e-12 * s0) || !(s0 > 0.0) || !isfinite(d)) bad = j0 + j + 1;
      else T[j * CBP + j] = sqrt(d);
    }
    __syncthreads();
    if (bad) break;
    const double piv = T[j * CBP + j];
    for (int i = j + 1 + threadIdx.x; i < b; i += blockDim.x) T[i * CBP + j] /= piv;
    __syncthreads();
    const int m = b - j - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int ii = e % m, ll = e / m;
      if (ll > ii) continue;
      T[(j + 1 + ii) * CBP + j + 1 + ll] -= T[(j + 1 + ii) * CBP + j] * T[(j + 1 + ll) * CBP + j];
    }
    __syncthreads();
  }
  if (bad) {
    if (threadIdx.x == 0) status[0] = bad;
    return;
  }
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int i = e % b, j = e / b;
    if (i >= j) A[(j0 + i) + (int64_t)(j0 + j) * k] = T[i * CBP + j];
  }
  __syncthreads();
  // inv(L11) by forward substitution, one thread per column j: reads the
  // lower triangle (never written here) and its own row j of the upper one
  if (threadIdx.x < b) {
    const int j = threadIdx.x;
    Vd[j] = 1.0 / T[j * CBP + j];
    for (int i = j + 1; i < b; ++i) {
      double sacc = -T[i * CBP + j] * Vd[j];
      for (int p = j + 1; p < i; ++p) sacc -= T[i * CBP + p] * T[j * CBP + p];
      T[j * CBP + i] = sacc / T[i * CBP + i];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int i = e % b, j = e / b;
    Linv[(j0 + i) + (int64_t)(j0 + j) * k] = i > j ? T[j * CBP + i] : (i == j ? Vd[i] : 0.0);
  }
}

// L21 = A21 inv(L11)^T for the rows [j0 + b + 64 blockIdx.x, +64)
__global__ void __launch_bounds__(256) k_chol_panel(double* __restrict__ A, int k, int j0, int b,
                                                    const double* __restrict__ Linv,
                                                    const int* __restrict__ status) {
  extern __shared__ double sm[];
  double* Vt = sm;               // Vt[t][s] = inv(L11)[t][s]
  double* R = sm + CB * CBP;     // R[r][s] = A21[r][s]
  if (status[0] != 0) return;
  const int r0 = j0 + b + blockIdx.x * CB;
  const int nr = min(CB, k - r0);
  for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
    const int i = e % CB, j = e / CB;
    Vt[i * CBP + j] = (i < b && j < b) ? Linv[(j0 + i) + (int64_t)(j0 + j) * k] : 0.0;
    R[i * CBP + j] = (i < nr && j < b) ? A[(r0 + i) + (int64_t)(j0 + j) * k] : 0.0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nr * b; e += blockDim.x) {
    const int r = e % nr, t = e / nr;
    double acc = 0.0;
    for (int sidx = 0; sidx <= t; ++sidx) acc = fma(R[r * CBP + sidx], Vt[t * CBP + sidx], acc);
    A[(r0 + r) + (int64_t)(j0 + t) * k] = acc;
  }
}

// A22 -= L21 L21^T on the tiles of the trailing lower triangle (64 x 64 each)
__global__ void __launch_bounds__(256) k_chol_update(double* __restrict__ A, int k, int j0, int b,
                                                     const int* __restrict__ status) {
  extern __shared__ double sm[];
  double* Li = sm;
  double* Ll = sm + CB * CBP;
  if (status[0] != 0) return;
  const int s0 = j0 + b;
  const int t = blockIdx.x;
  int bi = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while (bi * (bi + 1) / 2 > t) --bi;
  while ((bi + 1) * (bi + 2) / 2 <= t) ++bi;
  const int bj = t - bi * (bi + 1) / 2;
  const int i0 = s0 + bi * CB, l0 = s0 + bj * CB;
  for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
    const int r = e % CB, c = e / CB;
    Li[r * CBP + c] = (i0 + r < k && c < b) ? A[(i0 + r) + (int64_t)(j0 + c) * k] : 0.0;
    Ll[r * CBP + c] = (l0 + r < k && c < b) ? A[(l0 + r) + (int64_t)(j0 + c) * k] : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int c = 0; c < b; ++c) {
    double a[4], bb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = Li[(ty + 16 * u) * CBP + c];
      bb[u] = Ll[(tx + 16 * u) * CBP + c];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], bb[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty + 16 * u, l = l0 + tx + 16 * v;
      if (i < k && l < k && l <= i) A[i + (int64_t)l * k] -= acc[u][v];
    }
}

// Linv below the diagonal blocks: for block column J and 16 of its columns
// (blockIdx.y), X_I = -inv(L_II) sum_{J <= P < I} L_IP X_P for I = J+1, ...,
// with X_J = inv(L_JJ) (already in Linv).
__global__ void __launch_bounds__(256) k_chol_inv_offdiag(const double* __restrict__ L, int k,
                                                          double* __restrict__ Linv,
                                                          const int* __restrict__ status) {
  extern __shared__ double sm[];
  double* Lb = sm;                    // L_IP, then inv(L_II): 64 x 65
  double* Xp = sm + CB * CBP;         // X_P: 64 rows x 16 columns (stride 17)
  double* Acc = Xp + CB * 17;         // the sum: 64 x 16 (stride 17)
  if (status[0] != 0) return;
  const int nb = (k + CB - 1) / CB;
  const int J = blockIdx.x, c0 = J * CB + blockIdx.y * 16;
  if (c0 >= k || c0 >= (J + 1) * CB) return;
  const int nc = min(16, min(k, (J + 1) * CB) - c0);
  const int r = threadIdx.x % CB, cq = threadIdx.x / CB;   // row, 4-column quarter
  for (int I = J + 1; I < nb; ++I) {
    const int i0 = I * CB, ni = min(CB, k - i0);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int P = J; P < I; ++P) {
      const int p0 = P * CB, np = min(CB, k - p0);
      __syncthreads();
      for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
        const int a = e % CB, bcol = e / CB;
        Lb[a * CBP + bcol] = (a < ni && bcol < np) ? L[(i0 + a) + (int64_t)(p0 + bcol) * k] : 0.0;
      }
      for (int e = threadIdx.x; e < CB * 16; e += blockDim.x) {
        const int a = e % CB, cc = e / CB;
        Xp[a * 17 + cc] = (a < np && cc < nc) ? Linv[(p0 + a) + (int64_t)(c0 + cc) * k] : 0.0;
      }
      __syncthreads();
      for (int q = 0; q < np; ++q) {
        const double lv = Lb[r * CBP + q];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = fma(lv, Xp[q * 17 + 4 * cq + u], acc[u]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) Acc[r * 17 + 4 * cq + u] = acc[u];
    for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
      const int a = e % CB, bcol = e / CB;
      Lb[a * CBP + bcol] = (a < ni && bcol < ni) ? Linv[(i0 + a) + (int64_t)(i0 + bcol) * k] : 0.0;
    }
    __syncthreads();
    if (r < ni) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int cc = 4 * cq + u;
        if (cc >= nc) continue;
        double x = 0.0;
        for (int q = 0; q <= r; ++q) x = fma(Lb[r * CBP + q], Acc[q * 17 + cc], x);
        Linv[(i0 + r) + (int64_t)(c0 + cc) * k] = -x;
      }
    }
  }
}

__global__ void k_copy_diag(const double* __restrict__ A, int k, double* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) d[i] = A[i + (int64_t)i * k];
}

ttg_status cholesky_inv(ttg_op* op, double* S, double* Linv, int k, int* d_status) {
  if (k <= kCholSmall) {
    k_cholesky_inv<<<1, 1024, 0, op->stream>>>(S, Linv, k, d_status); TTG_COUNT();
    TTG_LAUNCHED(op);
    return TTG_OK;
  }
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    const int two = (int)(2 * kTileBytes);
    const int offd = (int)(kTileBytes + 2 * CB * 17 * sizeof(double));
    cudaError_t e1 = cudaFuncSetAttribute(k_chol_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, two);
    cudaError_t e2 = cudaFuncSetAttribute(k_chol_update, cudaFuncAttributeMaxDynamicSharedMemorySize, two);
    cudaError_t e3 = cudaFuncSetAttribute(k_chol_inv_offdiag,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, offd);
    attr = e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3;
  });
  if (attr != cudaSuccess) return TTG_CUDA_ERR;
  cudaStream_t st = op->stream;
  if (op->chol.bytes < (size_t)k * 8) TTG_TRY(op->chol.alloc((size_t)k * 8));
  double* diag0 = op->chol.as<double>();
  TTG_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), st));
  TTG_CUDA_TRY(cudaMemsetAsync(Linv, 0, (size_t)k * k * 8, st));
  k_copy_diag<<<(k + 255) / 256, 256, 0, st>>>(S, k, diag0); TTG_COUNT();
  TTG_LAUNCHED(op);
  for (int j0 = 0; j0 < k; j0 += CB) {
    const int b = std::min(CB, k - j0);
    k_chol_diag<<<1, 256, kTileBytes, st>>>(S, k, j0, b, diag0, Linv, d_status); TTG_COUNT();
    TTG_LAUNCHED(op);
    const int m = k - j0 - b;
    if (m <= 0) break;
    const int rb = (m + CB - 1) / CB;
    k_chol_panel<<<rb, 256, 2 * kTileBytes, st>>>(S, k, j0, b, Linv, d_status); TTG_COUNT();
    TTG_LAUNCHED(op);
    k_chol_update<<<rb * (rb + 1) / 2, 256, 2 * kTileBytes, st>>>(S, k, j0, b, d_status); TTG_COUNT();
    TTG_LAUNCHED(op);
  }
  const int nb = (k + CB - 1) / CB;
  k_chol_inv_offdiag<<<dim3(nb, CB / 16), 256,
                       kTileBytes + 2 * CB * 17 * sizeof(double), st>>>(S, k, Linv, d_status); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status syev_device(ttg_op* op, double* A, double* V, double* w, int k, int* d_status) {
  const int64_t kk = (int64_t)k * k;
  if (k <= 2048 && (int64_t)op->kk2.bytes >= kk * 8 &&
      (int64_t)op->scal.bytes >= (kScalJacobi + k) * (int64_t)sizeof(double)) {
    // the STHOSVD eigensolver with all k pairs (eig.cu): FP64 Householder on
    // a cluster of 8 CTAs, multisection, inverse iteration, Cholesky QR2.
    // FP64-accurate without refinement, and at k = 160 a little faster than
    // the FP32 QL + refinement below (about 1 ms per Rayleigh-Ritz pass).
    // A is overwritten.
    double* wtmp = op->scal.as<double>() + kScalJacobi;
    double* Vd = op->kk2.as<double>();
    TTG_TRY(sym_topk(op, A, k, k, wtmp, Vd, d_status));
    k_sort_eig<<<(k + 127) / 128, 128, 0, op->stream>>>(wtmp, Vd, w, V, k); TTG_COUNT();
    TTG_LAUNCHED(op);
    return TTG_OK;
  }
  // k > 2048: Householder + QL in FP32 (fast pipes), then two Ogita-Aishima
  // refinement steps (k x k GEMMs over all SMs) restore FP64 accuracy.
  const size_t need_f = (size_t)(2 * kk + 8 * (int64_t)k + 64) * sizeof(float);
  if ((int64_t)op->scal.bytes < (kScalJacobi + k) * (int64_t)sizeof(double) ||
      (int64_t)op->kk2.bytes < kk * 8 || op->kk3.bytes < need_f)
    return TTG_BAD_ARG;
  const size_t need_r = (size_t)(5 * kk + 8) * sizeof(double);
  if (op->eigbuf.bytes < need_r) TTG_TRY(op->eigbuf.alloc(need_r));
  cudaStream_t st = op->stream;
  double* wtmp = op->scal.as<double>() + kScalJacobi;
  double* Vd = op->kk2.as<double>();
  double* Gm = op->eigbuf.as<double>();
  double* AV = Gm + kk;
  double* Sm = AV + kk;
  double* E = Sm + kk;
  double* VE = E + kk;
  double* normA = VE + kk;
  float* Af = op->kk3.as<float>();
  float* Qf = Af + kk;
  float* wf = Qf + kk;
  k_symmetrize<<<64, 256, 0, st>>>(A, k); TTG_COUNT();
  TTG_LAUNCHED(op);
  k_frob2<<<1, 1024, 0, st>>>(A, kk, normA); TTG_COUNT();
  TTG_LAUNCHED(op);
  // FP32 stage: Af <- A; tridiagonalise + QL (scratch: vectors + reflectors)
  if (op->eigf.bytes < (size_t)(kk + 6 * (int64_t)k + 64) * sizeof(float))
    TTG_TRY(op->eigf.alloc((size_t)(kk + 6 * (int64_t)k + 64) * sizeof(float)));
  k_d2f_vec<<<64, 256, 0, st>>>(A, Af, kk); TTG_COUNT();
  TTG_LAUNCHED(op);
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_tridiag_ql<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    6 * 4096 * (int)sizeof(float));
  });
  if (attr_err != cudaSuccess) return TTG_CUDA_ERR;
  if (k > 4096) return TTG_BAD_ARG;
  k_tridiag_ql<float><<<1, 1024, 6 * k * sizeof(float), st>>>(Af, Qf, wf, k, d_status,
                                                              op->eigf.as<float>()); TTG_COUNT();
  TTG_LAUNCHED(op);
  k_f2d_vec<<<64, 256, 0, st>>>(Qf, Vd, kk); TTG_COUNT();
  TTG_LAUNCHED(op);
  const DOp Vt{Vd, (int64_t)k, 1, 0}, Vn{Vd, 1, (int64_t)k, 0}, An{A, 1, (int64_t)k, 0};
  for (int it = 0; it <= 2; ++it) {
    TTG_TRY(dgemm(st, k, k, k, 1, Vt, Vn, Gm, 1, k, 0, op->partial));           // G = V^T V
    TTG_TRY(dgemm(st, k, k, k, 1, An, Vn, AV, 1, k, 0, op->partial));           // A V
    TTG_TRY(dgemm(st, k, k, k, 1, Vt, DOp{AV, 1, (int64_t)k, 0}, Sm, 1, k, 0,
                  op->partial));                                                // S = V^T A V
    op->launches += 6;
    k_oa_step<<<1, 1024, 0, st>>>(Gm, Sm, k, normA, E, wtmp); TTG_COUNT();
    TTG_LAUNCHED(op);
    if (it == 2) break;                                                        // final lam only
    TTG_TRY(dgemm(st, k, k, k, 1, Vn, DOp{E, 1, (int64_t)k, 0}, VE, 1, k, 0, op->partial));
    op->launches += 2;
    k_add<<<64, 256, 0, st>>>(Vd, VE, kk); TTG_COUNT();
    TTG_LAUNCHED(op);
  }
  k_sort_eig<<<(k + 127) / 128, 128, 0, st>>>(wtmp, Vd, w, V, k); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status colmajor_to_rows(ttg_op* op, const double* src, int64_t ld_src, double* dst,
                            int64_t ld_dst, int64_t n, int k) {
  dim3 grid((unsigned)((n + 31) / 32), (unsigned)((k + 31) / 32));
  k_cm_to_rows<<<grid, dim3(32, 8), 0, op->stream>>>(src, ld_src, dst, ld_dst, n, k); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status rows_to_colmajor(ttg_op* op, const double* src, int64_t ld_src, double* dst,
                            int64_t ld_dst, int64_t n, int k) {
  dim3 grid((unsigned)((n + 31) / 32), (unsigned)((k + 31) / 32));
  k_rows_to_cm<<<grid, dim3(32, 8), 0, op->stream>>>(src, ld_src, dst, ld_dst, n, k); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status lanczos_step(ttg_op* op, double* v, double* v0, const double* hv, double* ab, int it) {
  k_lanczos_step<<<1, 1024, 0, op->stream>>>(v, v0, hv, op->n, op->ld, ab, it); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status normalize(ttg_op* op, double* v) {
  k_normalize<<<1, 1024, 0, op->stream>>>(v, op->n, op->ld); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status fermi(ttg_op* op, const double* eig, int k, double ne, double kT, int max_iter,
                 double* occ, double* out) {
  k_fermi<<<1, 256, 0, op->stream>>>(eig, k, ne, kT, max_iter, occ, out); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

}  // namespace ttg

// ------------------------------------------------------------------------
// Allocation-free Gram matrix.
//
// Some callers cannot call cudaMalloc: code running inside a memory pool or
// an arena that owns all device memory, plugins whose host forbids driver
// allocations after start-up, or callers that must not synchronise the
// device (cudaMalloc/cudaFree can).  ttg_gram_noalloc computes the same
// S = X^T Y as ttg_gram with caller-owned inputs and outputs, and keeps its
// split-K partial sums in the fixed array below instead of allocating.
//
// The array is a file-scope __device__ variable: every GPU that loads this
// library holds kNoAllocScratchDoubles doubles (16 MiB) until the process
// exits.  All calls share it and it keeps the last call's contents; each call
// overwrites every partial it later reads, so nothing needs clearing.  Calls
// whose work overlaps on the GPU (different streams, or host threads) race on
// it and must be serialised by the caller.
// The host cannot use the array's name as a device address, so the first call
// on each device looks the address up with cudaGetSymbolAddress (with that
// device current) and caches it.  With lazy module loading that lookup also
// loads this library's device code and commits the array, so the first call
// belongs at start-up, before any stream capture and before the caller's
// no-allocation phase.  The cache lives as long as the process: a
// cudaDeviceReset of the device invalidates it, and this entry point must
// not be called on that device afterwards.
namespace {

constexpr int64_t kNoAllocScratchDoubles = 2 * 1024 * 1024;
__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices] = {};
std::mutex g_noalloc_mu;

ttg_status noalloc_scratch(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return TTG_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "ttg: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      cudaGetLastError();
      return TTG_CUDA_ERR;
    }
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return TTG_OK;
}

}  // namespace

extern "C" ttg_status ttg_gram_noalloc(const double* x_dev, const double* y_dev, int64_t n,
                                       int32_t k, int64_t ld, double* s_dev, void* stream) {
  if (!x_dev || !y_dev || !s_dev || n <= 0 || k <= 0 || ld < k) return TTG_BAD_ARG;
  const int64_t kk = (int64_t)k * k;
  if (kk > kNoAllocScratchDoubles) {
    fprintf(stderr, "ttg_gram_noalloc: k = %d needs %lld scratch doubles, the maximum is %lld\n",
            k, (long long)kk, (long long)kNoAllocScratchDoubles);
    return TTG_BAD_ARG;
  }
  double* scratch = nullptr;
  TTG_TRY(noalloc_scratch(&scratch));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int tp = (k + ttg::TM - 1) / ttg::TM, tq = (k + ttg::TN - 1) / ttg::TN;
  const int tiles = tp * tq;
  int64_t nsplit = (2 * 152 + tiles - 1) / tiles;
  nsplit = std::min<int64_t>(nsplit, (n + 255) / 256);
  nsplit = std::min<int64_t>(nsplit, kNoAllocScratchDoubles / kk);
  if (nsplit < 1) nsplit = 1;
  const int64_t rows = (n + nsplit - 1) / nsplit;
  ttg::k_gram_tn<<<dim3(tp, tq, (unsigned)nsplit), 256, 0, st>>>(x_dev, y_dev, n, k, ld, rows,
                                                                scratch, 0); TTG_COUNT();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return TTG_CUDA_ERR;
  ttg::k_reduce_splits<<<(unsigned)std::min<int64_t>((kk + 255) / 256, 1024), 256, 0, st>>>(
      scratch, (int)nsplit, kk, s_dev, 0); TTG_COUNT();
  e = cudaGetLastError();
  return e == cudaSuccess ? TTG_OK : TTG_CUDA_ERR;
}
