// Self-consistent-field glue on the device, FP64: Tucker compression of grid
// fields (STHOSVD), Tucker reconstruction, LDA exchange-correlation, weighted
// grid integrals and linear combinations (Anderson mixing), and the update of
// the Hamiltonian's values when the effective potential changes.
//
//   ttg_tucker_sthosvd     TuckerMPI::STHOSVD as called by the reference
//                          (tensor/TensorUtils.cc:245-264, main.cc:951-955,
//                          dft/ProjectHamiltonianSparse.cc:1113-1118):
//                          sequential truncation, mode by mode, of the
//                          eigen-decomposition of the mode Gram matrix.
//   ttg_tucker_reconstruct core x1 U1 x2 U2 x3 U3 (Tucker::ttm chain).
//   ttg_grid_lda           KSDFTPotential::computeLDAExchangePot /
//                          computeLDACorrelationPot (dft/KSDFTPotential.cc:
//                          127-267) and the energy density of
//                          KSDFTEnergyFunctional::computeLDAExchangeCorrelationEnergy
//                          (dft/KSDFTEnergyFunctional.cc:27-56).
//   ttg_grid_integrate     compute3DIntegral (KSDFTEnergyFunctional.cc:169-192)
//                          with the separable J*w weights; also the weighted
//                          inner products of AndersonMixing::computeMixingConstants
//                          (dft/AndersonMixing.cc:150-265).
//   ttg_grid_lincomb       sum_m c_m f_m (optionally |.|): AndersonMixing::
//                          computeRhoIn (dft/AndersonMixing.cc:267-316).
//
// Fields are x-fastest n1 x n2 x n3 arrays in device memory owned by the
// caller.  The mode products and Gram matrices are one strided-batched GEMM
// kernel (FP64 in and out, double-FP32 arithmetic on the FP32 pipe) with a
// fixed-order split-K reduction in FP64 (bitwise reproducible).

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "ttg_internal.cuh"

namespace ttg {
namespace {

constexpr int DM = 64, DN = 64, DK = 16;
constexpr int64_t kNumSMs = 152;

// C[z] (+)= A[z] B[z] over a K range, in df64; split s of z_total =
// batch*splits writes its partial to part + s*... when part != nullptr.
// sym: the product is symmetric (a Gram matrix); tiles strictly above the
// diagonal are skipped and filled by k_mirror_upper afterwards.
__global__ void __launch_bounds__(256) k_dgemm(int M, int N, int K, int splits, DOp A, DOp B,
                                               double* C, int64_t c_rs, int64_t c_cs, int64_t c_bs,
                                               double* part, int sym) {
  __shared__ float sAh[DK][DM + 1], sAl[DK][DM + 1];
  __shared__ float sBh[DK][DN + 1], sBl[DK][DN + 1];
  const int zz = blockIdx.z;
  const int z = zz / splits, sp = zz % splits;
  const int kchunk = (K + splits - 1) / splits;
  const int kbeg = sp * kchunk, kend = min(K, kbeg + kchunk);
  int mt = blockIdx.y, nt = blockIdx.x;
  if (sym) {          // blockIdx.x enumerates the tiles on and below the diagonal
    const int i = blockIdx.x;
    mt = (int)((sqrt(8.0 * i + 1.0) - 1.0) * 0.5);
    while ((mt + 1) * (mt + 2) / 2 <= i) ++mt;
    while (mt * (mt + 1) / 2 > i) --mt;
    nt = i - mt * (mt + 1) / 2;
  }
  const int m0 = mt * DM, n0 = nt * DN;
  const double* Ab = A.p + (int64_t)z * A.bs;
  const double* Bb = B.p + (int64_t)z * B.bs;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const bool a_mfast = (A.rs == 1), b_nfast = (B.cs == 1);
  F2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = F2{0.f, 0.f};
  for (int kb = kbeg; kb < kend; kb += DK) {
    for (int e = threadIdx.x; e < DK * DM; e += 256) {
      int mm, kk;
      if (a_mfast) { mm = e % DM; kk = e / DM; } else { kk = e % DK; mm = e / DK; }
      const int gm = m0 + mm, gk = kb + kk;
      const F2 av = to_f2((gm < M && gk < kend) ? Ab[(int64_t)gm * A.rs + (int64_t)gk * A.cs] : 0.0);
      sAh[kk][mm] = av.h;
      sAl[kk][mm] = av.l;
      int nn, kk2;
      if (b_nfast) { nn = e % DN; kk2 = e / DN; } else { kk2 = e % DK; nn = e / DK; }
      const int gn = n0 + nn, gk2 = kb + kk2;
      const F2 bv = to_f2((gn < N && gk2 < kend) ? Bb[(int64_t)gk2 * B.rs + (int64_t)gn * B.cs] : 0.0);
      sBh[kk2][nn] = bv.h;
      sBl[kk2][nn] = bv.l;
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < DK; ++t) {
      F2 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = F2{sAh[t][ty + 16 * u], sAl[t][ty + 16 * u]};
        b[u] = F2{sBh[t][tx + 16 * u], sBl[t][tx + 16 * u]};
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
      const int m = m0 + ty + 16 * u, n = n0 + tx + 16 * v;
      if (m >= M || n >= N) continue;
      const double r = (double)acc[u][v].h + (double)acc[u][v].l;
      if (part) part[((int64_t)zz * M + m) * N + n] = r;
      else C[(int64_t)z * c_bs + (int64_t)m * c_rs + (int64_t)n * c_cs] = r;
    }
}

__global__ void k_dgemm_reduce(const double* __restrict__ part, int batch, int splits, int M,
                               int N, double* C, int64_t c_rs, int64_t c_cs, int64_t c_bs,
                               int sym) {
  const int64_t total = (int64_t)batch * M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(e / ((int64_t)M * N));
    const int64_t r = e - (int64_t)z * M * N;
    const int m = (int)(r / N), n = (int)(r - (int64_t)m * N);
    if (sym && n > m) continue;
    double s = 0.0;
    for (int sp = 0; sp < splits; ++sp) s += part[(((int64_t)z * splits + sp) * M + m) * N + n];
    C[(int64_t)z * c_bs + (int64_t)m * c_rs + (int64_t)n * c_cs] = s;
  }
}

// C[m, n] = C[n, m] for n > m (square, batch 1).
__global__ void k_mirror_upper(double* C, int M, int64_t c_rs, int64_t c_cs) {
  const int64_t total = (int64_t)M * M;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(e / M), n = (int)(e - (int64_t)m * M);
    if (n > m) C[(int64_t)m * c_rs + (int64_t)n * c_cs] = C[(int64_t)n * c_rs + (int64_t)m * c_cs];
  }
}

// Sum of a batch of matrices: out = sum_z in[z] (fixed order).
__global__ void k_sum_batches(const double* __restrict__ in, int batch, int64_t size,
                              double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < size;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < batch; ++z) s += in[(int64_t)z * size + e];
    out[e] = s;
  }
}

int gblocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 16);
}

}  // namespace

// Generic FP64 GEMM with automatic split-K when the output is small.
ttg_status dgemm(cudaStream_t st, int M, int N, int K, int batch, DOp A, DOp B, double* C,
                 int64_t c_rs, int64_t c_cs, int64_t c_bs, DevBuf& scratch, bool sym) {
  if (M <= 0 || N <= 0 || batch <= 0) return TTG_OK;
  if (sym && (M != N || batch != 1)) return TTG_BAD_ARG;
  const int64_t tm = (M + DM - 1) / DM, tn = (N + DN - 1) / DN;
  const int64_t tiles = sym ? tm * (tm + 1) / 2 : tm * tn * batch;
  // split K so that the CTAs fill the SMs evenly (FP64 throughput is per
  // SM: the busiest SM sets the time)
  int splits = 1;
  if (tiles < kNumSMs && K > 4 * DK) {
    splits = (int)std::min<int64_t>(kNumSMs / tiles, (K + 4 * DK - 1) / (4 * DK));
    splits = std::max(1, std::min(splits, 256));
  }
  if ((int64_t)batch * splits > 65535) return TTG_BAD_ARG;
  dim3 grid(sym ? (unsigned)tiles : (unsigned)tn, sym ? 1u : (unsigned)tm, batch * splits);
  if (grid.y > 65535) return TTG_BAD_ARG;
  double* part = nullptr;
  if (splits > 1) {
    const size_t need = (size_t)batch * splits * M * N * sizeof(double);
    if (scratch.bytes < need) TTG_TRY(scratch.alloc(need));
    part = scratch.as<double>();
  }
  k_dgemm<<<grid, 256, 0, st>>>(M, N, K, splits, A, B, C, c_rs, c_cs, c_bs, part, sym ? 1 : 0); TTG_COUNT();
  if (cudaGetLastError() != cudaSuccess) return TTG_CUDA_ERR;
  if (splits > 1) {
    k_dgemm_reduce<<<gblocks((int64_t)batch * M * N), 256, 0, st>>>(part, batch, splits, M, N, C,
                                                                     c_rs, c_cs, c_bs, sym ? 1 : 0); TTG_COUNT();
    if (cudaGetLastError() != cudaSuccess) return TTG_CUDA_ERR;
  }
  if (sym) {
    k_mirror_upper<<<gblocks((int64_t)M * M), 256, 0, st>>>(C, M, c_rs, c_cs); TTG_COUNT();
    if (cudaGetLastError() != cudaSuccess) return TTG_CUDA_ERR;
  }
  return TTG_OK;
}

namespace {

// Mode-d product of an x-fastest tensor (n0, n1, n2) with Mmat (p x n_d,
// row-major): mode d of the result has size p.
ttg_status mode_product(cudaStream_t st, const double* T, const int* n, int d, const double* Mmat,
                        int p, double* out, DevBuf& scratch) {
  const int64_t n0 = n[0], n1 = n[1], n2 = n[2];
  if (d == 0) {
    // out (p x n1 n2) = M (p x n0) T_(0) (n0 x n1 n2)
    return dgemm(st, p, (int)(n1 * n2), (int)n0, 1, DOp{Mmat, (int64_t)n0, 1, 0},
                 DOp{T, 1, n0, 0}, out, 1, p, 0, scratch);
  }
  if (d == 1) {
    // per slab l: out_l (n0 x p) = T_l (n0 x n1) M^T (n1 x p)
    return dgemm(st, (int)n0, p, (int)n1, (int)n2, DOp{T, 1, n0, n0 * n1},
                 DOp{Mmat, 1, n1, 0}, out, 1, n0, n0 * p, scratch);
  }
  // out (n0 n1 x p) = T (n0 n1 x n2) M^T (n2 x p)
  return dgemm(st, (int)(n0 * n1), p, (int)n2, 1, DOp{T, 1, n0 * n1, 0}, DOp{Mmat, 1, n2, 0}, out,
               1, n0 * n1, 0, scratch);
}

// Gram matrix of mode d, G (n_d x n_d) column-major.
ttg_status mode_gram(cudaStream_t st, const double* T, const int* n, int d, double* G,
                     DevBuf& scratch, DevBuf& scratch2) {
  const int64_t n0 = n[0], n1 = n[1], n2 = n[2];
  if (d == 0)
    return dgemm(st, (int)n0, (int)n0, (int)(n1 * n2), 1, DOp{T, 1, n0, 0}, DOp{T, n0, 1, 0}, G,
                 1, n0, 0, scratch, true);
  if (d == 2)
    return dgemm(st, (int)n2, (int)n2, (int)(n0 * n1), 1, DOp{T, n0 * n1, 1, 0},
                 DOp{T, 1, n0 * n1, 0}, G, 1, n2, 0, scratch, true);
  // mode 1: sum over slabs l of T_l^T T_l (n1 x n1), T_l = (n0 x n1) column-major
  const size_t need = (size_t)n2 * n1 * n1 * sizeof(double);
  if (scratch2.bytes < need) TTG_TRY(scratch2.alloc(need));
  TTG_TRY(dgemm(st, (int)n1, (int)n1, (int)n0, (int)n2, DOp{T, n0, 1, n0 * n1},
                DOp{T, 1, n0, n0 * n1}, scratch2.as<double>(), 1, n1, n1 * n1, scratch));
  k_sum_batches<<<gblocks(n1 * n1), 256, 0, st>>>(scratch2.as<double>(), (int)n2, n1 * n1, G); TTG_COUNT();
  return cudaGetLastError() == cudaSuccess ? TTG_OK : TTG_CUDA_ERR;
}

// Perdew-Zunger LDA with the reference's constants
// (dft/KSDFTEnergyFunctional.h:76-82).
constexpr double kGamma = -0.1423, kBeta1 = 1.0529, kBeta2 = 0.3334, kA = 0.0311, kB = -0.048,
                 kC = 0.002, kD = -0.0116;

__global__ void k_lda(const double* __restrict__ rho, int64_t n, double* __restrict__ v,
                      double* __restrict__ e, int accumulate_v) {
  const double exch_c = -(3.0 / 4.0) * cbrt(3.0 / M_PI);
  const double c0 = cbrt(3.0 / (4.0 * M_PI));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double r = rho[i];
    const double cr = cbrt(r);
    // exchange: potential (4/3) c rho^(1/3), energy density c rho^(4/3)
    const double vx = exch_c * (4.0 / 3.0) * cr;
    const double ex = exch_c * r * cr;
    // correlation potential as the reference computes it (KSDFTPotential.cc:
    // 254-265): rs = (3/(4 pi rho))^(1/3) and, for rs < 1, a (2D - C) rs / 33
    // term where the Perdew-Zunger form has / 3.
    double vc;
    const double rsv = cbrt(3.0 / (4.0 * M_PI * r));
    if (rsv >= 1.0) {
      const double sq = sqrt(rsv);
      const double den = 1.0 + kBeta1 * sq + kBeta2 * rsv;
      vc = kGamma * (1.0 + (7.0 / 6.0) * kBeta1 * sq + (4.0 / 3.0) * kBeta2 * rsv) / (den * den);
    } else {
      const double lr = log(rsv);
      vc = kA * lr + (kB - kA / 3.0) + (2.0 / 3.0) * kC * rsv * lr + (2.0 * kD - kC) * rsv / 33.0;
    }
    // correlation energy density (KSDFTEnergyFunctional.cc:37-52)
    const double rs = c0 / (cr + 1.0e-12);
    double ec;
    if (rs >= 1.0) {
      ec = kGamma / (1.0 + kBeta1 * sqrt(rs) + kBeta2 * rs);
    } else {
      const double lr = log(rs);
      ec = kA * lr + kB + kC * rs * lr + kD * rs;
    }
    if (v) v[i] = (accumulate_v ? v[i] : 0.0) + vx + vc;
    if (e) e[i] = ex + ec * r;
  }
}

// partial[b] = sum over block b of f*g*wx*wy*wz (g may be null)
__global__ void k_wsum(const double* __restrict__ f, const double* __restrict__ g,
                       const double* __restrict__ wx, const double* __restrict__ wy,
                       const double* __restrict__ wz, int n0, int n1, int n2,
                       double* __restrict__ partial) {
  __shared__ double red[32];
  const int64_t total = (int64_t)n0 * n1 * n2;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % n0);
    const int64_t yz = i / n0;
    const int y = (int)(yz % n1), z = (int)(yz / n1);
    double v = f[i] * wx[x] * wy[y] * wz[z];
    if (g) v *= g[i];
    s += v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}

__global__ void k_sum_partials(const double* partial, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += partial[i];
    *out = s;
  }
}

// out[i,j,l] = sum_a c_a fx[a,i] fy[a,j] fz[a,l] (+ out when accumulate):
// superposition of separable per-atom fields (the atomic densities of
// InitialGuess::initializeRhoFromRadiusFile, dft/InitialGuess.cc:573-681, and
// the Gaussian-well local potential).
__global__ void k_cp_sum(int na, const double* __restrict__ c, const double* __restrict__ fx,
                         const double* __restrict__ fy, const double* __restrict__ fz, int n0,
                         int n1, int n2, double* __restrict__ out, int accumulate) {
  const int64_t total = (int64_t)n0 * n1 * n2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % n0);
    const int64_t yz = i / n0;
    const int y = (int)(yz % n1), z = (int)(yz / n1);
    double s = accumulate ? out[i] : 0.0;
    for (int a = 0; a < na; ++a)
      s = fma(c[a] * fx[(int64_t)a * n0 + x], fy[(int64_t)a * n1 + y] * fz[(int64_t)a * n2 + z], s);
    out[i] = s;
  }
}

// Electrostatic potential of Gaussian ionic charges, exact:
// out += -sum_a Z_a erf(|r - R_a| / w) / |r - R_a|  (limit 2 Z_a / (sqrt(pi) w) at 0)
__global__ void k_ion_potential(int na, const double* __restrict__ pos, const double* __restrict__ z,
                                double w, const double* __restrict__ gx,
                                const double* __restrict__ gy, const double* __restrict__ gz,
                                int n0, int n1, int n2, double* __restrict__ out) {
  const int64_t total = (int64_t)n0 * n1 * n2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % n0);
    const int64_t yz = i / n0;
    const int y = (int)(yz % n1), zz = (int)(yz / n1);
    double s = 0.0;
    for (int a = 0; a < na; ++a) {
      const double dx = gx[x] - pos[3 * a], dy = gy[y] - pos[3 * a + 1], dz = gz[zz] - pos[3 * a + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      s += z[a] * (r > 1e-10 ? erf(r / w) / r : 2.0 / (sqrt(M_PI) * w));
    }
    out[i] -= s;
  }
}

// M_t[q, a] = sum_q' exp(-alpha_t (x_q - x_q')^2) WU[q', a]   grid (q, K), block r
__global__ void k_gauss_apply(const double* __restrict__ alpha, const double* __restrict__ x,
                              int nq, const double* __restrict__ WU, int r, double* __restrict__ M) {
  extern __shared__ double ex[];
  const int q = blockIdx.x, t = blockIdx.y;
  const double at = alpha[t], xq = x[q];
  for (int p = threadIdx.x; p < nq; p += blockDim.x) {
    const double d = xq - x[p];
    ex[p] = exp(-at * d * d);
  }
  __syncthreads();
  for (int a = threadIdx.x; a < r; a += blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nq; ++p) s = fma(ex[p], WU[p + (int64_t)a * nq], s);
    M[((int64_t)t * r + a) * nq + q] = s;     // [t][a][q]: column-major q x r per term
  }
}

// Partial sums of <G, U> for one term: part[blockIdx.x] (deterministic: the
// host adds the partials in order).
__global__ void __launch_bounds__(256) k_dot_part(const double* __restrict__ G,
                                                  const double* __restrict__ U, int64_t n,
                                                  double* __restrict__ part) {
  __shared__ double red[8];
  double sum = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    sum = fma(G[e], U[e], sum);
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < 8; ++w) tot += red[w];
    part[blockIdx.x] = tot;
  }
}

__global__ void k_diag_sum(const double* __restrict__ A, int n, double* out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += A[i + (int64_t)i * n];
    *out = s;
  }
}

constexpr int kMaxLinTerms = 24;   // Anderson depth 10: 2 x 11 fields
struct LinTerms {
  const double* f[kMaxLinTerms];
  double c[kMaxLinTerms];
};

__global__ void k_lincomb(LinTerms t, int nt, int64_t n, double* out, int take_abs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int m = 0; m < nt; ++m) s += t.c[m] * t.f[m][i];
    out[i] = take_abs ? fabs(s) : s;
  }
}

}  // namespace
}  // namespace ttg

using namespace ttg;

namespace {

struct Stream {
  cudaStream_t s = nullptr;
  bool own = false;
  explicit Stream(void* st) {
    if (st) {
      s = static_cast<cudaStream_t>(st);
    } else {
      cudaStreamCreateWithFlags(&s, cudaStreamDefault);
      own = true;
    }
  }
  ~Stream() {
    if (own) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }
};

}  // namespace

extern "C" {

ttg_status ttg_tucker_sthosvd(ttg_op* op, const double* t_dev, const int32_t* dims, double eps,
                              const int32_t* max_ranks, int32_t* ranks_out, double* core_dev,
                              double* u0_dev, double* u1_dev, double* u2_dev) {
  if (!op || !t_dev || !dims || !ranks_out || !core_dev || !u0_dev || !u1_dev || !u2_dev)
    return TTG_BAD_ARG;
  int n[3] = {dims[0], dims[1], dims[2]};
  for (int d = 0; d < 3; ++d)
    if (n[d] <= 0 || n[d] > 2048) return TTG_BAD_ARG;
  cudaStream_t st = op->stream;
  const int64_t total = (int64_t)n[0] * n[1] * n[2];
  DevBuf norm;
  DevBuf& A = op->sth_a;
  DevBuf& B = op->sth_b;
  DevBuf& part = op->sth_part;
  DevBuf& part2 = op->sth_part2;
  if (A.bytes < (size_t)total * 8) TTG_TRY(A.alloc(total * 8));
  if (B.bytes < (size_t)total * 8) TTG_TRY(B.alloc(total * 8));
  TTG_TRY(norm.alloc(4096 * 8));
  TTG_CUDA_TRY(cudaMemcpyAsync(A.p, t_dev, total * 8, cudaMemcpyDeviceToDevice, st));
  // ||T||^2 for the truncation threshold eps^2 ||T||^2 / 3 per mode
  {
    std::vector<double> ones(4096, 1.0);
    DevBuf w1;
    TTG_TRY(w1.alloc(4096 * 8));
    TTG_CUDA_TRY(cudaMemcpyAsync(w1.p, ones.data(), 4096 * 8, cudaMemcpyHostToDevice, st));
    const int nb = 1024;
    k_wsum<<<nb, 256, 0, st>>>(A.as<double>(), A.as<double>(), w1.as<double>(), w1.as<double>(),
                               w1.as<double>(), n[0], n[1], n[2], norm.as<double>()); TTG_COUNT();
    k_sum_partials<<<1, 32, 0, st>>>(norm.as<double>(), nb, norm.as<double>() + 2048); TTG_COUNT();
    TTG_LAUNCHED(op);
    TTG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  double norm2 = 0.0;
  TTG_CUDA_TRY(cudaMemcpy(&norm2, norm.as<double>() + 2048, 8, cudaMemcpyDeviceToHost));
  const double thr = eps * eps * norm2 / 3.0;
  double* U[3] = {u0_dev, u1_dev, u2_dev};
  int cur[3] = {n[0], n[1], n[2]};
  for (int d = 0; d < 3; ++d) {
    const int nd = cur[d];
    const int rcap = std::min(nd, (max_ranks && max_ranks[d] > 0) ? (int)max_ranks[d] : nd);
    const size_t kk = (size_t)nd * nd * 8;
    if (op->kk0.bytes < kk) TTG_TRY(op->kk0.alloc(kk));
    TTG_TRY(mode_gram(st, A.as<double>(), cur, d, op->kk0.as<double>(), part, part2));
    // trace of the Gram = sum of all eigenvalues
    k_diag_sum<<<1, 256, 0, st>>>(op->kk0.as<double>(), nd, norm.as<double>() + 2049); TTG_COUNT();
    TTG_LAUNCHED(op);
    // the rcap largest eigenpairs in FP64 (the truncation needs eigenvectors whose
    // eigenvalues are many orders below the largest one)
    double* wdev = norm.as<double>() + 1024;
    TTG_TRY(sym_topk(op, op->kk0.as<double>(), nd, rcap, wdev, U[d], op->status.as<int>()));
    std::vector<double> w(rcap + 1);
    int stat = 0;
    TTG_CUDA_TRY(cudaMemcpyAsync(w.data(), wdev, rcap * 8, cudaMemcpyDeviceToHost, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(&w[rcap], norm.as<double>() + 2049, 8, cudaMemcpyDeviceToHost, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(&stat, op->status.p, 4, cudaMemcpyDeviceToHost, st));
    TTG_CUDA_TRY(cudaStreamSynchronize(st));
    if (stat) return TTG_NOT_CONVERGED;
    const double trace = w[rcap];
    // smallest r whose discarded eigenvalues sum to <= thr
    int r = rcap;   // eps 0: fixed rank
    double kept = 0.0;
    for (int i = 0; i < rcap && thr > 0.0; ++i) {
      kept += std::max(w[i], 0.0);
      if (trace - kept <= thr) {
        r = i + 1;
        break;
      }
    }
    ranks_out[d] = r;
    // project: A <- A x_d U_d^T
    TTG_TRY(mode_product(st, A.as<double>(), cur, d, U[d], r, B.as<double>(), part));
    std::swap(A.p, B.p);
    std::swap(A.bytes, B.bytes);
    cur[d] = r;
  }
  TTG_CUDA_TRY(cudaMemcpyAsync(core_dev, A.p, (size_t)cur[0] * cur[1] * cur[2] * 8,
                               cudaMemcpyDeviceToDevice, st));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  return TTG_OK;
}

ttg_status ttg_tucker_reconstruct(const double* core_dev, const int32_t* ranks,
                                  const double* u0_dev, const double* u1_dev,
                                  const double* u2_dev, const int32_t* dims, double* out_dev,
                                  void* stream) {
  if (!core_dev || !ranks || !dims || !out_dev || !u0_dev || !u1_dev || !u2_dev)
    return TTG_BAD_ARG;
  Stream S(stream);
  const double* U[3] = {u0_dev, u1_dev, u2_dev};
  int cur[3] = {ranks[0], ranks[1], ranks[2]};
  DevBuf a, b, part;
  const int64_t big = (int64_t)std::max(dims[0], ranks[0]) * std::max(dims[1], ranks[1]) *
                      std::max(dims[2], ranks[2]);
  TTG_TRY(a.alloc(big * 8));
  TTG_TRY(b.alloc(big * 8));
  TTG_CUDA_TRY(cudaMemcpyAsync(a.p, core_dev, (size_t)cur[0] * cur[1] * cur[2] * 8,
                               cudaMemcpyDeviceToDevice, S.s));
  // U_d is n_d x r_d column-major = (r_d x n_d)^T; as the row-major p x n matrix
  // M of mode_product we need M[i, a] = U[i + n*a]: rows i, stride 1 between a
  // -> pass through dgemm directly here
  for (int d = 0; d < 3; ++d) {
    const int nd = dims[d], rd = cur[d];
    const int64_t n0 = cur[0], n1 = cur[1], n2 = cur[2];
    ttg_status s;
    if (d == 0)
      s = dgemm(S.s, nd, (int)(n1 * n2), rd, 1, DOp{U[0], 1, nd, 0}, DOp{a.as<double>(), 1, n0, 0},
                b.as<double>(), 1, nd, 0, part);
    else if (d == 1)
      s = dgemm(S.s, (int)n0, nd, rd, (int)n2, DOp{a.as<double>(), 1, n0, n0 * n1},
                DOp{U[1], nd, 1, 0}, b.as<double>(), 1, n0, n0 * nd, part);
    else
      s = dgemm(S.s, (int)(n0 * n1), nd, rd, 1, DOp{a.as<double>(), 1, n0 * n1, 0},
                DOp{U[2], nd, 1, 0}, b.as<double>(), 1, n0 * n1, 0, part);
    if (s != TTG_OK) return s;
    std::swap(a.p, b.p);
    std::swap(a.bytes, b.bytes);
    cur[d] = nd;
  }
  TTG_CUDA_TRY(cudaMemcpyAsync(out_dev, a.p, (size_t)dims[0] * dims[1] * dims[2] * 8,
                               cudaMemcpyDeviceToDevice, S.s));
  TTG_CUDA_TRY(cudaStreamSynchronize(S.s));
  return TTG_OK;
}

ttg_status ttg_hartree_energy(int32_t K, const double* alpha, const double* omega,
                              const int32_t* ranks, const double* G, const int32_t* nq,
                              const double* xq0, const double* xq1, const double* xq2,
                              const double* wq0, const double* wq1, const double* wq2,
                              const double* u0, const double* u1, const double* u2,
                              double* energy) {
  if (K <= 0 || !alpha || !omega || !ranks || !G || !nq || !energy) return TTG_BAD_ARG;
  const double* xs[3] = {xq0, xq1, xq2};
  const double* ws[3] = {wq0, wq1, wq2};
  const double* us[3] = {u0, u1, u2};
  int r[3];
  for (int d = 0; d < 3; ++d) {
    r[d] = ranks[d];
    if (r[d] <= 0 || nq[d] <= 0 || !xs[d] || !ws[d] || !us[d]) return TTG_BAD_ARG;
  }
  Stream S(nullptr);
  DevBuf dalpha, core, x[3], wu[3], M[3], Kd[3], t0, t1, scratch, res;
  TTG_TRY(dalpha.alloc(K * 8));
  TTG_CUDA_TRY(cudaMemcpyAsync(dalpha.p, alpha, K * 8, cudaMemcpyHostToDevice, S.s));
  const int64_t ncore = (int64_t)r[0] * r[1] * r[2];
  TTG_TRY(core.alloc(ncore * 8));
  TTG_CUDA_TRY(cudaMemcpyAsync(core.p, G, ncore * 8, cudaMemcpyHostToDevice, S.s));
  for (int d = 0; d < 3; ++d) {
    const int q = nq[d];
    std::vector<double> h((size_t)q * r[d]);
    for (int a = 0; a < r[d]; ++a)
      for (int p = 0; p < q; ++p) h[p + (size_t)a * q] = ws[d][p] * us[d][p + (size_t)a * q];
    TTG_TRY(x[d].alloc(q * 8));
    TTG_TRY(wu[d].alloc(h.size() * 8));
    TTG_TRY(M[d].alloc((size_t)K * r[d] * q * 8));
    TTG_TRY(Kd[d].alloc((size_t)K * r[d] * r[d] * 8));
    TTG_CUDA_TRY(cudaMemcpyAsync(x[d].p, xs[d], q * 8, cudaMemcpyHostToDevice, S.s));
    TTG_CUDA_TRY(cudaMemcpyAsync(wu[d].p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, S.s));
    k_gauss_apply<<<dim3(q, K), 128, q * 8, S.s>>>(dalpha.as<double>(), x[d].as<double>(), q,
                                                    wu[d].as<double>(), r[d], M[d].as<double>()); TTG_COUNT();
    TTG_CUDA_TRY(cudaGetLastError());
    // K_t[a, a'] = sum_q WU[q, a] M_t[q, a']  (batched over t), column-major r x r
    TTG_TRY(dgemm(S.s, r[d], r[d], q, K, DOp{wu[d].as<double>(), q, 1, 0},
                  DOp{M[d].as<double>(), 1, q, (int64_t)r[d] * q}, Kd[d].as<double>(), 1, r[d],
                  (int64_t)r[d] * r[d], scratch));
  }
  // E_t = <G, G x1 Kx_t x2 Ky_t x3 Kz_t>, term by term as three GEMMs
  // (H = G x3 Kz_t, T = Kx_t H, U = T x2 Ky_t, slab by slab) and a dot product
  const int64_t nab = (int64_t)r[0] * r[1];
  constexpr int kParts = 256;
  DevBuf hbuf, tbuf;
  TTG_TRY(hbuf.alloc((size_t)ncore * 8));
  TTG_TRY(tbuf.alloc((size_t)ncore * 8));
  TTG_TRY(res.alloc((size_t)K * kParts * 8));
  double* H = hbuf.as<double>();
  double* T = tbuf.as<double>();
  for (int t = 0; t < K; ++t) {
    const double* kx = Kd[0].as<double>() + (int64_t)t * r[0] * r[0];
    const double* ky = Kd[1].as<double>() + (int64_t)t * r[1] * r[1];
    const double* kz = Kd[2].as<double>() + (int64_t)t * r[2] * r[2];
    // H[(a, b), c'] = sum_c G[(a, b), c] Kz[c, c']
    TTG_TRY(dgemm(S.s, (int)nab, r[2], r[2], 1, DOp{core.as<double>(), 1, nab, 0},
                  DOp{kz, 1, r[2], 0}, H, 1, nab, 0, scratch));
    // T[a', (b, c')] = sum_a Kx[a', a] H[a, (b, c')]
    TTG_TRY(dgemm(S.s, r[0], (int)((int64_t)r[1] * r[2]), r[0], 1, DOp{kx, 1, r[0], 0},
                  DOp{H, 1, r[0], 0}, T, 1, r[0], 0, scratch));
    // U[a', b', c'] = sum_b T[a', b, c'] Ky[b, b'], one batch per slab c' (into H)
    TTG_TRY(dgemm(S.s, r[0], r[1], r[1], r[2], DOp{T, 1, r[0], nab}, DOp{ky, 1, r[1], 0}, H, 1,
                  r[0], nab, scratch));
    k_dot_part<<<kParts, 256, 0, S.s>>>(core.as<double>(), H, ncore,
                                        res.as<double>() + (int64_t)t * kParts); TTG_COUNT();
    TTG_CUDA_TRY(cudaGetLastError());
  }
  std::vector<double> e((size_t)K * kParts);
  TTG_CUDA_TRY(cudaMemcpyAsync(e.data(), res.p, e.size() * 8, cudaMemcpyDeviceToHost, S.s));
  TTG_CUDA_TRY(cudaStreamSynchronize(S.s));
  double s = 0.0;
  for (int t = 0; t < K; ++t) {
    double et = 0.0;
    for (int c = 0; c < kParts; ++c) et += e[(size_t)t * kParts + c];
    s += omega[t] * et;
  }
  *energy = 0.5 * s;
  return TTG_OK;
}

ttg_status ttg_grid_lda(const double* rho_dev, int64_t n, double* v_dev, double* e_dev,
                        int32_t accumulate_v, void* stream) {
  if (!rho_dev || n <= 0) return TTG_BAD_ARG;
  Stream S(stream);
  k_lda<<<gblocks(n), 256, 0, S.s>>>(rho_dev, n, v_dev, e_dev, accumulate_v); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  return TTG_OK;
}

ttg_status ttg_grid_integrate(const double* f_dev, const double* g_dev, const int32_t* dims,
                              const double* wx_dev, const double* wy_dev, const double* wz_dev,
                              double* result, void* stream) {
  if (!f_dev || !dims || !wx_dev || !wy_dev || !wz_dev || !result) return TTG_BAD_ARG;
  Stream S(stream);
  DevBuf part;
  const int nb = 1024;
  TTG_TRY(part.alloc((nb + 1) * 8));
  k_wsum<<<nb, 256, 0, S.s>>>(f_dev, g_dev, wx_dev, wy_dev, wz_dev, dims[0], dims[1], dims[2],
                              part.as<double>()); TTG_COUNT();
  k_sum_partials<<<1, 32, 0, S.s>>>(part.as<double>(), nb, part.as<double>() + nb); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  TTG_CUDA_TRY(cudaMemcpyAsync(result, part.as<double>() + nb, 8, cudaMemcpyDeviceToHost, S.s));
  TTG_CUDA_TRY(cudaStreamSynchronize(S.s));
  return TTG_OK;
}

ttg_status ttg_grid_cp_sum(int32_t nterms, const double* coef_dev, const double* fx_dev,
                           const double* fy_dev, const double* fz_dev, const int32_t* dims,
                           double* out_dev, int32_t accumulate, void* stream) {
  if (nterms < 0 || !dims || !out_dev || (nterms > 0 && (!coef_dev || !fx_dev || !fy_dev || !fz_dev)))
    return TTG_BAD_ARG;
  Stream S(stream);
  const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
  k_cp_sum<<<gblocks(n), 256, 0, S.s>>>(nterms, coef_dev, fx_dev, fy_dev, fz_dev, dims[0], dims[1],
                                        dims[2], out_dev, accumulate); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  return TTG_OK;
}

ttg_status ttg_grid_ion_potential(int32_t natoms, const double* pos_dev, const double* z_dev,
                                  double width, const double* gx_dev, const double* gy_dev,
                                  const double* gz_dev, const int32_t* dims, double* out_dev,
                                  void* stream) {
  if (natoms < 0 || !dims || !out_dev || !(width > 0) || !gx_dev || !gy_dev || !gz_dev)
    return TTG_BAD_ARG;
  Stream S(stream);
  const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
  k_ion_potential<<<gblocks(n), 256, 0, S.s>>>(natoms, pos_dev, z_dev, width, gx_dev, gy_dev, gz_dev,
                                               dims[0], dims[1], dims[2], out_dev); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  return TTG_OK;
}

ttg_status ttg_grid_lincomb(int32_t nterms, const double* const* fields_dev, const double* coef,
                            int64_t n, double* out_dev, int32_t take_abs, void* stream) {
  if (nterms <= 0 || nterms > kMaxLinTerms || !fields_dev || !coef || !out_dev || n <= 0) return TTG_BAD_ARG;
  Stream S(stream);
  LinTerms t{};
  for (int m = 0; m < nterms; ++m) {
    t.f[m] = fields_dev[m];
    t.c[m] = coef[m];
  }
  k_lincomb<<<gblocks(n), 256, 0, S.s>>>(t, nterms, n, out_dev, take_abs); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  return TTG_OK;
}

}  // extern "C"
