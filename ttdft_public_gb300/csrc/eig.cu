// Largest r eigenpairs of a symmetric n x n matrix in FP64: the mode Gram
// matrices of the sequentially truncated HOSVD (TuckerMPI::STHOSVD as used
// at main.cc:951-955 and ProjectHamiltonianSparse.cc:1113-1118), whose
// eigenvalues span ~14 orders of magnitude, so that an FP32 eigensolver
// cannot resolve the truncation subspace.
//
// FP64 runs at a small fraction of the FP32 rate on this GPU, so no stage is
// left to a single SM:
//
//  1. Householder tridiagonalisation A = Q T Q^T by one cluster of kCluster
//     CTAs.  A stays in global memory (L2-resident); per column j every CTA
//     forms the reflector v_j redundantly, each CTA computes its rows of
//     p = tau B v, the pieces are exchanged through distributed shared
//     memory, and each CTA applies B <- B - v w^T - w v^T to its own columns.
//     Two cluster barriers per column.
//  2. Eigenvalues by multisection on Sturm counts: one warp per eigenvalue,
//     one CTA per warp, 32 points per round (bisection would take 52 rounds
//     to reach FP64 resolution, multisection 11).
//  3. Eigenvectors of T by inverse iteration (tridiagonal LU with partial
//     pivoting, three passes; equal eigenvalues are separated by a small
//     shift perturbation as in LAPACK's dstein), then u = Q z by applying
//     the stored reflectors in reverse order: one CTA per eigenvector.
//  4. Orthonormalisation U <- U L^-T with U^T U = L L^T, twice (Cholesky QR2;
//     the inverse-iteration vectors are already orthonormal to ~1e-8 or
//     better), with a Gram-Schmidt fallback if a Cholesky pivot fails.

#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <mutex>

#include "ttg_internal.cuh"

namespace cg = cooperative_groups;

namespace ttg {
namespace {

constexpr int kCluster = 8;
constexpr int kTrThreads = 512;
constexpr int kVecThreads = 256;
constexpr int kMaxN = 2048;

__device__ double cta_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;
}

__device__ __forceinline__ int chunk_begin(int m, int q) { return (int)(((int64_t)m * q) / kCluster); }

// Stage 1.  A (n x n column-major, symmetric) is overwritten; outputs the
// diagonal d, off-diagonal e (e[i] couples i and i+1), tau and the reflectors
// Vr (column j holds v_j in rows j+1..n-1).
__global__ void __cluster_dims__(kCluster, 1, 1) __launch_bounds__(kTrThreads)
    k_tridiag_cluster(double* __restrict__ A, int n, double* __restrict__ d,
                      double* __restrict__ e, double* __restrict__ tau,
                      double* __restrict__ Vr) {
  cg::cluster_group cl = cg::this_cluster();
  const int q = (int)cl.block_rank();
  extern __shared__ double sm[];
  double* v = sm;                                   // n
  double* p = v + n;                                // n
  double* pch = p + n;                              // n / kCluster + 1
  double* part = pch + n / kCluster + 1;            // kTrThreads
  __shared__ double red[32];
  __shared__ double s_alpha, s_tau;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kTrThreads / 32;
  for (int j = 0; j + 2 < n; ++j) {
    const int m = n - j - 1;
    const double* col = A + (j + 1) + (int64_t)j * n;
    double ss = 0.0;
    for (int r = tid; r < m; r += kTrThreads) {
      const double x = __ldcg(col + r);
      v[r] = x;
      ss += x * x;
    }
    ss = cta_sum(ss, red);
    if (tid == 0) {
      const double x0 = v[0];
      const double nrm = sqrt(ss);
      const double alpha = x0 >= 0.0 ? -nrm : nrm;
      const double vn2 = ss - x0 * x0 + (x0 - alpha) * (x0 - alpha);
      s_alpha = alpha;
      s_tau = vn2 > 0.0 ? 2.0 / vn2 : 0.0;
      v[0] = x0 - alpha;
      if (q == 0) {
        d[j] = __ldcg(A + j + (int64_t)j * n);
        e[j] = vn2 > 0.0 ? alpha : x0;
        tau[j] = s_tau;
      }
    }
    __syncthreads();
    const double tj = s_tau;
    if (q == 0)
      for (int r = tid; r < m; r += kTrThreads) Vr[(j + 1 + r) + (int64_t)j * n] = v[r];
    if (tj == 0.0) continue;                       // same decision on every CTA
    // rows [rb, re) of p = tau B v, B = A[j+1:, j+1:]
    const int rb = chunk_begin(m, q), re = chunk_begin(m, q + 1), cnt = re - rb;
    if (cnt > 0) {
      const int nsub = kTrThreads / cnt;
      const int rr = tid % cnt, sub = tid / cnt;
      if (sub < nsub) {
        const double* brow = A + (j + 1 + rb + rr) + (int64_t)(j + 1) * n;
        double acc = 0.0;
        for (int c = sub; c < m; c += nsub) acc = fma(__ldcg(brow + (int64_t)c * n), v[c], acc);
        part[sub * cnt + rr] = acc;
      }
      __syncthreads();
      if (tid < cnt) {
        double s = 0.0;
        for (int u = 0; u < nsub; ++u) s += part[u * cnt + tid];
        pch[tid] = tj * s;
      }
    }
    cl.sync();
    for (int qq = 0; qq < kCluster; ++qq) {
      const int b0 = chunk_begin(m, qq), b1 = chunk_begin(m, qq + 1);
      const double* rem = cl.map_shared_rank(pch, qq);
      for (int r = b0 + tid; r < b1; r += kTrThreads) p[r] = rem[r - b0];
    }
    __syncthreads();
    double vp = 0.0;
    for (int r = tid; r < m; r += kTrThreads) vp += v[r] * p[r];
    vp = cta_sum(vp, red);
    const double K = 0.5 * tj * vp;
    for (int r = tid; r < m; r += kTrThreads) p[r] -= K * v[r];
    __syncthreads();
    // own columns [rb, re) of B: B[:, c] -= v w_c + w v_c
    for (int c = rb + warp; c < re; c += kWarps) {
      double* bc = A + (j + 1) + (int64_t)(j + 1 + c) * n;
      const double vc = v[c], wc = p[c];
      for (int r = lane; r < m; r += 32) __stcg(bc + r, __ldcg(bc + r) - v[r] * wc - p[r] * vc);
    }
    cl.sync();
  }
  if (q == 0 && tid == 0) {
    for (int j = (n >= 2 ? n - 2 : 0); j < n; ++j) {
      d[j] = __ldcg(A + j + (int64_t)j * n);
      e[j] = (j + 1 < n) ? __ldcg(A + (j + 1) + (int64_t)j * n) : 0.0;
      tau[j] = 0.0;
    }
  }
}

__device__ int sturm_count(const double* d, const double* e2, int n, double x) {
  int cnt = 0;
  double qv = d[0] - x;
  cnt += qv < 0.0;
  for (int i = 1; i < n; ++i) {
    if (fabs(qv) < 1e-300) qv = -1e-300;
    qv = d[i] - x - e2[i - 1] / qv;
    cnt += qv < 0.0;
  }
  return cnt;
}

// Stage 2: eigenvalue b (descending order) per CTA of one warp.
__global__ void __launch_bounds__(32) k_tridiag_multisect(const double* __restrict__ d,
                                                          const double* __restrict__ e, int n,
                                                          double* __restrict__ w) {
  extern __shared__ double sm[];
  double* sd = sm;
  double* se2 = sm + n;
  const int lane = threadIdx.x, b = blockIdx.x;
  double lo = 1e300, hi = -1e300;
  for (int i = lane; i < n; i += 32) {
    sd[i] = d[i];
    se2[i] = (i + 1 < n) ? e[i] * e[i] : 0.0;
    const double rad = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - rad);
    hi = fmax(hi, d[i] + rad);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __syncwarp();
  const double pad = 4.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + 1e-300;
  lo -= pad;
  hi += pad;
  const int target = n - 1 - b;                 // ascending index
  for (int round = 0; round < 40; ++round) {
    if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + 1e-300) break;
    const double x = lo + (hi - lo) * (double)(lane + 1) / 33.0;
    const int cnt = sturm_count(sd, se2, n, x);
    const unsigned above = __ballot_sync(0xffffffffu, cnt > target);
    const double xprev = __shfl_up_sync(0xffffffffu, x, 1);
    if (above == 0u) {
      lo = __shfl_sync(0xffffffffu, x, 31);
    } else {
      const int L = __ffs(above) - 1;
      const double nhi = __shfl_sync(0xffffffffu, x, L);
      const double nlo = __shfl_sync(0xffffffffu, xprev, L);
      hi = nhi;
      if (L > 0) lo = nlo;
    }
  }
  if (lane == 0) w[b] = 0.5 * (lo + hi);
}

// Stage 3: eigenvector b: inverse iteration on T, then u = Q z.  Dynamic
// shared memory: d, e, dg, u1, u2, z (6n doubles).
__global__ void __launch_bounds__(kVecThreads) k_tridiag_vectors(
    const double* __restrict__ d, const double* __restrict__ e, const double* __restrict__ tau,
    const double* __restrict__ Vr, const double* __restrict__ w, int n, double* __restrict__ U) {
  extern __shared__ double sm[];
  double* sd = sm;
  double* se = sd + n;
  double* dg = se + n;
  double* u1 = dg + n;
  double* u2 = u1 + n;
  double* z = u2 + n;
  __shared__ double red[32];
  __shared__ double s_shift;
  const int tid = threadIdx.x, b = blockIdx.x;
  double tn = 0.0;
  for (int i = tid; i < n; i += kVecThreads) {
    sd[i] = d[i];
    se[i] = e[i];
    tn = fmax(tn, fabs(d[i]) + fabs(e[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0));
  }
  for (int o = 16; o > 0; o >>= 1) tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
  if ((tid & 31) == 0) red[tid >> 5] = tn;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int i = 0; i < kVecThreads / 32; ++i) t = fmax(t, red[i]);
    // separate (nearly) equal eigenvalues: w is descending
    const double pert = 10.0 * DBL_EPSILON * t + 1e-300;
    double s = w[0];
    for (int i = 1; i <= b; ++i) {
      const double wi = w[i];
      s = (s - wi < pert) ? s - pert : wi;
    }
    s_shift = s;
    red[0] = t;
  }
  __syncthreads();
  const double lam = s_shift, tnorm = red[0];
  if (tid == 0) {
    const double guard = DBL_EPSILON * tnorm + 1e-300;
    uint32_t seed = 0x9e3779b9u * (uint32_t)(b + 1);
    for (int i = 0; i < n; ++i) {
      seed = seed * 1664525u + 1013904223u;
      z[i] = 0.5 + (double)(seed >> 8) * (1.0 / 16777216.0);
    }
    for (int pass = 0; pass < 3; ++pass) {
      double a = sd[0] - lam, bb = (n > 1 ? se[0] : 0.0), c = 0.0;
      double zc = z[0];
      for (int i = 0; i + 1 < n; ++i) {
        const double sub = se[i];
        const double na = sd[i + 1] - lam, nb = (i + 2 < n ? se[i + 1] : 0.0);
        double zn = z[i + 1];
        if (fabs(a) >= fabs(sub)) {
          const double mlt = (a != 0.0 ? sub / a : 0.0);
          dg[i] = a; u1[i] = bb; u2[i] = c;
          a = na - mlt * bb; bb = nb - mlt * c; c = 0.0;
          zn -= mlt * zc;
        } else {
          const double mlt = a / sub;
          dg[i] = sub; u1[i] = na; u2[i] = nb;
          const double t = zc; zc = zn; zn = t - mlt * zn;
          a = bb - mlt * na; bb = c - mlt * nb; c = 0.0;
        }
        z[i] = zc;
        zc = zn;
      }
      dg[n - 1] = a;
      z[n - 1] = zc;
      double nrm = 0.0;
      for (int i = n - 1; i >= 0; --i) {
        double vv = z[i];
        if (i + 1 < n) vv -= u1[i] * z[i + 1];
        if (i + 2 < n) vv -= u2[i] * z[i + 2];
        const double piv = fabs(dg[i]) > guard ? dg[i] : (dg[i] >= 0.0 ? guard : -guard);
        z[i] = vv / piv;
        nrm = fmax(nrm, fabs(z[i]));
      }
      const double inv = 1.0 / nrm;
      for (int i = 0; i < n; ++i) z[i] *= inv;
    }
  }
  __syncthreads();
  // u = H_0 H_1 ... H_{n-3} z
  for (int j = n - 3; j >= 0; --j) {
    const double tj = tau[j];
    if (tj == 0.0) continue;
    const int m = n - j - 1;
    const double* vj = Vr + (j + 1) + (int64_t)j * n;
    double dot = 0.0;
    for (int r = tid; r < m; r += kVecThreads) dot += vj[r] * z[j + 1 + r];
    dot = cta_sum(dot, red) * tj;
    for (int r = tid; r < m; r += kVecThreads) z[j + 1 + r] -= dot * vj[r];
    __syncthreads();
  }
  double nn = 0.0;
  for (int i = tid; i < n; i += kVecThreads) nn += z[i] * z[i];
  nn = cta_sum(nn, red);
  const double inv = 1.0 / sqrt(nn);
  for (int i = tid; i < n; i += kVecThreads) U[(int64_t)b * n + i] = z[i] * inv;
}

// Fallback orthonormalisation: classical Gram-Schmidt with one
// reorthogonalisation pass, column by column, one CTA.
__global__ void __launch_bounds__(1024) k_cgs2(double* __restrict__ U, int n, int r,
                                               double* __restrict__ coef) {
  __shared__ double red[32];
  for (int j = 0; j < r; ++j) {
    double* uj = U + (int64_t)j * n;
    for (int pass = 0; pass < 2; ++pass) {
      // coef[i] = u_i . u_j for i < j: one warp per i
      for (int i = threadIdx.x >> 5; i < j; i += blockDim.x >> 5) {
        const double* ui = U + (int64_t)i * n;
        double s = 0.0;
        for (int t = threadIdx.x & 31; t < n; t += 32) s += ui[t] * uj[t];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) coef[i] = s;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < n; t += blockDim.x) {
        double s = uj[t];
        for (int i = 0; i < j; ++i) s -= coef[i] * U[(int64_t)i * n + t];
        uj[t] = s;
      }
      __syncthreads();
    }
    double nn = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) nn += uj[t] * uj[t];
    nn = cta_sum(nn, red);
    const double inv = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) uj[t] *= inv;
    __syncthreads();
  }
}

__global__ void k_symmetrize_lower(double* A, int n) {
  const int64_t total = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i % n), c = (int)(i / n);
    if (r > c) {
      const double s = 0.5 * (A[i] + A[c + (int64_t)r * n]);
      A[i] = s;
      A[c + (int64_t)r * n] = s;
    }
  }
}

}  // namespace

ttg_status sym_topk(ttg_op* op, double* A, int n, int r, double* w, double* U, int* d_status) {
  if (r < 1 || r > n || n > kMaxN) return TTG_BAD_ARG;
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_tridiag_vectors, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    6 * kMaxN * (int)sizeof(double));
  });
  if (attr_err != cudaSuccess) return TTG_CUDA_ERR;
  const int64_t nn = (int64_t)n * n;
  const size_t need = (size_t)(nn + 3 * (int64_t)n + 2 * (int64_t)r * r + (int64_t)n * r + 64) *
                      sizeof(double);
  if (op->eigbuf.bytes < need) TTG_TRY(op->eigbuf.alloc(need));
  cudaStream_t st = op->stream;
  double* Vr = op->eigbuf.as<double>();
  double* dd = Vr + nn;
  double* ee = dd + n;
  double* tt = ee + n;
  double* S = tt + n;
  double* Li = S + (int64_t)r * r;
  double* U2 = Li + (int64_t)r * r;
  k_symmetrize_lower<<<64, 256, 0, st>>>(A, n); TTG_COUNT();
  TTG_LAUNCHED(op);
  const size_t sm_tr = (size_t)(2 * n + n / kCluster + 1 + kTrThreads) * sizeof(double);
  k_tridiag_cluster<<<kCluster, kTrThreads, sm_tr, st>>>(A, n, dd, ee, tt, Vr); TTG_COUNT();
  TTG_LAUNCHED(op);
  k_tridiag_multisect<<<r, 32, 2 * n * sizeof(double), st>>>(dd, ee, n, w); TTG_COUNT();
  TTG_LAUNCHED(op);
  k_tridiag_vectors<<<r, kVecThreads, 6 * n * sizeof(double), st>>>(dd, ee, tt, Vr, w, n, U); TTG_COUNT();
  TTG_LAUNCHED(op);
  // Cholesky QR2: U <- U L^-T with U^T U = L L^T
  for (int pass = 0; pass < 2; ++pass) {
    TTG_TRY(dgemm(st, r, r, n, 1, DOp{U, (int64_t)n, 1, 0}, DOp{U, 1, (int64_t)n, 0}, S, 1, r, 0,
                  op->partial));
    TTG_TRY(cholesky_inv(op, S, Li, r, d_status));
    int stat = 0;
    TTG_CUDA_TRY(cudaMemcpyAsync(&stat, d_status, 4, cudaMemcpyDeviceToHost, st));
    TTG_CUDA_TRY(cudaStreamSynchronize(st));
    if (stat != 0) {
      k_cgs2<<<1, 1024, 0, st>>>(U, n, r, S); TTG_COUNT();
      TTG_LAUNCHED(op);
      TTG_CUDA_TRY(cudaMemsetAsync(d_status, 0, 4, st));
      break;
    }
    TTG_TRY(dgemm(st, n, r, r, 1, DOp{U, 1, (int64_t)n, 0}, DOp{Li, (int64_t)r, 1, 0}, U2, 1, n, 0,
                  op->partial));
    TTG_CUDA_TRY(cudaMemcpyAsync(U, U2, (size_t)n * r * sizeof(double), cudaMemcpyDeviceToDevice,
                                 st));
    op->launches += 4;
  }
  return TTG_OK;
}

}  // namespace ttg
