// Tucker-mode contractions on the tensor cores: the density build
// (ProjectHamiltonianSparse::computeRhoOut, dft/ProjectHamiltonianSparse.cc:
// 911-1221, per-state ttm chain :1051-1074) and the Hartree kernel expansion
// (KSDFTPotential::computeHartreePotNew, dft/KSDFTPotential.cc:269-340; factor
// integrals :440-599; per-term ttm + daxpy :601-658).
//
// Both are chains of mode products, written here as strided, batched GEMMs
//   C[z](m, n) = alpha * sum_k A[z](m, k) B[z](k, n) (+ beta C)
// with FP32 operands and a three-term TF32 split on the tensor cores:
//   A B ~= A_hi B_hi + A_hi B_lo + A_lo B_hi,  X_hi = tf32(X), X_lo = tf32(X - X_hi)
// which keeps FP32-level accuracy (the dropped A_lo B_lo term is ~2^-22
// relative).  Accumulation is FP32.
//
// Hartree: all K expansion terms go through ONE launch for the dominant
// mode-3 product: V[(i,j), l] = sum_{(t,c)} Q_t[(i,j), c] * (w_t Fz_t[l, c]),
// i.e. the K terms are stacked along the contraction dimension, so V is
// written once instead of being updated K times (the reference's per-term
// daxpy, KSDFTPotential.cc:641-654).
//
// Density: the last mode product is fused with the square-and-weight
// reduction over states: rho[i,j,l] = sum_s 2 f_s psi_s[i,j,l]^2, so the
// per-state orbitals psi_s on the nodal grid are never written to HBM.

#include <algorithm>
#include <cmath>
#include <vector>

#include "ttg_internal.cuh"

namespace ttg {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, PAD = 4;
constexpr int NTHR = 128;

struct Operand {
  const float* p;
  int64_t rs;   // stride of the first index (row)
  int64_t cs;   // stride of the second index (col)
  int64_t bs;   // batch stride
  int div = 1;  // batch z uses offset (z / div) * bs
};

__device__ __forceinline__ uint32_t tf32_of(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_of(x);
  lo = tf32_of(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum Epi { EPI_STORE = 0, EPI_SQSUM = 1 };

// Epilogue parameters for EPI_SQSUM: output column n = p * S + s (S states,
// S % 32 == 0), rho[m * rho_rs + p * rho_cs] += sum_s w[s] * C(m, n)^2.
struct SqSum {
  float* rho;
  const float* w;
  int S;
  int64_t rho_rs, rho_cs;
};

template <int EPI>
__global__ void __launch_bounds__(NTHR) k_gemm_x3(int M, int N, int K, Operand A, Operand B,
                                                  float* C, int64_t c_rs, int64_t c_cs,
                                                  int64_t c_bs, float alpha, float beta,
                                                  SqSum sq) {
  __shared__ float sA[2][BK][BM + PAD];
  __shared__ float sB[2][BK][BN + PAD];
  const int z = blockIdx.z;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const float* Ab = A.p + (int64_t)(z / A.div) * A.bs;
  const float* Bb = B.p + (int64_t)(z / B.div) * B.bs;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int wm = (warp / 2) * 32, wn = (warp % 2) * 32;
  const int g = lane >> 2, t = lane & 3;
  // global -> register staging: 8 elements of A and 8 of B per thread
  const bool a_mfast = (A.rs == 1);
  const bool b_nfast = (B.cs == 1);
  float ra[8], rb[8];
  auto load_tiles = [&](int k0) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + u * NTHR;           // 0..1023
      int mm, kk;
      if (a_mfast) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      const int gm = m0 + mm, gk = k0 + kk;
      ra[u] = (gm < M && gk < K) ? __ldg(Ab + (int64_t)gm * A.rs + (int64_t)gk * A.cs) : 0.f;
      int nn, kb;
      if (b_nfast) { nn = e % BN; kb = e / BN; } else { kb = e % BK; nn = e / BK; }
      const int gn = n0 + nn, gkb = k0 + kb;
      rb[u] = (gn < N && gkb < K) ? __ldg(Bb + (int64_t)gkb * B.rs + (int64_t)gn * B.cs) : 0.f;
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + u * NTHR;
      int mm, kk;
      if (a_mfast) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      sA[buf][kk][mm] = ra[u];
      int nn, kb;
      if (b_nfast) { nn = e % BN; kb = e / BN; } else { kb = e % BK; nn = e / BK; }
      sB[buf][kb][nn] = rb[u];
    }
  };
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  const int nk = (K + BK - 1) / BK;
  load_tiles(0);
  store_tiles(0);
  __syncthreads();
  for (int kt = 0; kt < nk; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < nk) load_tiles((kt + 1) * BK);
#pragma unroll
    for (int k8 = 0; k8 < BK; k8 += 8) {
      uint32_t ahi[2][4], alo[2][4], bhi[4][2], blo[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int mb = wm + i * 16;
        split_tf32(sA[buf][k8 + t][mb + g], ahi[i][0], alo[i][0]);
        split_tf32(sA[buf][k8 + t][mb + g + 8], ahi[i][1], alo[i][1]);
        split_tf32(sA[buf][k8 + t + 4][mb + g], ahi[i][2], alo[i][2]);
        split_tf32(sA[buf][k8 + t + 4][mb + g + 8], ahi[i][3], alo[i][3]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nb = wn + j * 8;
        split_tf32(sB[buf][k8 + t][nb + g], bhi[j][0], blo[j][0]);
        split_tf32(sB[buf][k8 + t + 4][nb + g], bhi[j][1], blo[j][1]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          mma_tf32(acc[i][j], alo[i], bhi[j]);
          mma_tf32(acc[i][j], ahi[i], blo[j]);
          mma_tf32(acc[i][j], ahi[i], bhi[j]);
        }
    }
    if (kt + 1 < nk) {
      store_tiles(buf ^ 1);
    }
    __syncthreads();
  }
  if constexpr (EPI == EPI_STORE) {
    float* Cb = C + (int64_t)z * c_bs;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + wm + i * 16 + g + (q >= 2 ? 8 : 0);
          const int n = n0 + wn + j * 8 + 2 * t + (q & 1);
          if (m < M && n < N) {
            float* o = Cb + (int64_t)m * c_rs + (int64_t)n * c_cs;
            *o = alpha * acc[i][j][q] + (beta != 0.f ? beta * *o : 0.f);
          }
        }
  } else {
    // each warp's 32 columns belong to one p (S % 32 == 0, tile aligned)
    const int nbase = n0 + wn;
    if (nbase >= N) return;
    const int p = nbase / sq.S;
    const int s0 = nbase - p * sq.S;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int q2 = 0; q2 < 2; ++q2) {
            const float c = alpha * acc[i][j][h * 2 + q2];
            const int s = s0 + j * 8 + 2 * t + q2;
            v = fmaf(sq.w[s] * c, c, v);
          }
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        const int m = m0 + wm + i * 16 + g + h * 8;
        if (t == 0 && m < M) atomicAdd(sq.rho + (int64_t)m * sq.rho_rs + (int64_t)p * sq.rho_cs, v);
      }
  }
}

// Fx_t[i, a] = sum_q wq[q] exp(-alpha_t (x_i - xq_q)^2) U[q, a], FP64 on the
// CUDA cores (KSDFTPotential.cc:509-523), stored FP32 row-major [t][i][a].
__global__ void k_expansion_factor(const double* __restrict__ alpha, int K,
                                   const double* __restrict__ x, int nx,
                                   const double* __restrict__ xq, const double* __restrict__ wq,
                                   int nq, const double* __restrict__ U, int r,
                                   float* __restrict__ F, const double* __restrict__ scale) {
  const int t = blockIdx.z;
  const int i = blockIdx.y;
  const double at = alpha[t];
  const double xi = x[i];
  extern __shared__ double e[];
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const double d = xi - xq[q];
    e[q] = wq[q] * exp(-at * d * d);
  }
  __syncthreads();
  const double sc = scale ? scale[t] : 1.0;
  for (int a = threadIdx.x; a < r; a += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s += e[q] * U[q + (int64_t)a * nq];
    F[((int64_t)t * nx + i) * r + a] = (float)(sc * s);
  }
}

__global__ void k_d2f(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (float)s[i];
}

__global__ void k_f2d(const float* __restrict__ s, double* __restrict__ d, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (double)s[i];
}

// density: FP64 row-major block (n x ld) -> FP32 [row][s] with S padded columns
__global__ void k_block_to_f32(const double* __restrict__ X, int64_t n, int k, int64_t ld,
                               float* __restrict__ out, int S) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * S;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / S;
    const int s = (int)(e - r * S);
    out[e] = s < k ? (float)X[r * ld + s] : 0.f;
  }
}

int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 16);
}

template <int EPI>
ttg_status gemm(cudaStream_t st, int M, int N, int K, int batch, Operand A, Operand B, float* C,
                int64_t c_rs, int64_t c_cs, int64_t c_bs, float alpha, float beta, SqSum sq,
                int64_t* launches) {
  if (M <= 0 || N <= 0 || K <= 0 || batch <= 0) return TTG_OK;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
  if (grid.y > 65535 || grid.z > 65535) return TTG_BAD_ARG;
  k_gemm_x3<EPI><<<grid, NTHR, 0, st>>>(M, N, K, A, B, C, c_rs, c_cs, c_bs, alpha, beta, sq); TTG_COUNT();
  if (launches) (*launches)++;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TTG_OK : TTG_CUDA_ERR;
}

struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T> T* get(int64_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<int64_t>(n, 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ptrs.push_back(p);
    return reinterpret_cast<T*>(p);
  }
};

}  // namespace
}  // namespace ttg

using namespace ttg;

extern "C" {

ttg_status ttg_density(ttg_op* op, const ttg_block* X, const double* occ_host, int32_t rx,
                       int32_t ry, int32_t rz, int32_t nx, int32_t ny, int32_t nz,
                       const double* ux, const double* uy, const double* uz, double* rho_host) {
  if (!op || !X || X->op != op || !occ_host || !ux || !uy || !uz || !rho_host) return TTG_BAD_ARG;
  if ((int64_t)rx * ry * rz != op->n || nx <= 0 || ny <= 0 || nz <= 0) return TTG_BAD_ARG;
  const int k = X->k;
  const int S = (k + 31) / 32 * 32;   // states padded to whole warps
  cudaStream_t st = op->stream;
  Scratch sc;
  const int64_t n = op->n;
  float* Xf = sc.get<float>(n * S);
  float* Ux = sc.get<float>((int64_t)nx * rx);
  float* Uy = sc.get<float>((int64_t)ny * ry);
  float* Uz = sc.get<float>((int64_t)nz * rz);
  float* w = sc.get<float>(S);
  float* P1 = sc.get<float>((int64_t)ry * rz * nx * S);
  float* P2 = sc.get<float>((int64_t)rz * ny * nx * S);
  float* rho = sc.get<float>((int64_t)nx * ny * nz);
  double* stage = sc.get<double>(std::max<int64_t>({(int64_t)nx * rx, (int64_t)ny * ry,
                                                    (int64_t)nz * rz, (int64_t)nx * ny * nz}));
  if (!Xf || !Ux || !Uy || !Uz || !w || !P1 || !P2 || !rho || !stage) return TTG_OOM;
  k_block_to_f32<<<blocks_for(n * S), 256, 0, st>>>(X->x.as<double>(), n, k, op->ld, Xf, S); TTG_COUNT();
  TTG_LAUNCHED(op);
  // basis values at the nodes, column-major (nodes x rank)
  const double* hs[3] = {ux, uy, uz};
  float* ds[3] = {Ux, Uy, Uz};
  const int64_t cnt[3] = {(int64_t)nx * rx, (int64_t)ny * ry, (int64_t)nz * rz};
  for (int d = 0; d < 3; ++d) {
    TTG_CUDA_TRY(cudaMemcpyAsync(stage, hs[d], cnt[d] * 8, cudaMemcpyHostToDevice, st));
    k_d2f<<<blocks_for(cnt[d]), 256, 0, st>>>(stage, ds[d], cnt[d]); TTG_COUNT();
    TTG_LAUNCHED(op);
  }
  std::vector<float> wh(S, 0.f);
  for (int s = 0; s < k; ++s) wh[s] = (float)(2.0 * occ_host[s]);
  TTG_CUDA_TRY(cudaMemcpyAsync(w, wh.data(), S * 4, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemsetAsync(rho, 0, (int64_t)nx * ny * nz * 4, st));
  SqSum none{nullptr, nullptr, 1, 0, 0};
  // 1) P1[bc][i][s] = sum_a Ux[i,a] X[(a + rx*bc)][s]    batch over bc
  TTG_TRY(gemm<EPI_STORE>(st, nx, S, rx, ry * rz, Operand{Ux, 1, nx, 0},
                          Operand{Xf, S, 1, (int64_t)rx * S}, P1, S, 1, (int64_t)nx * S, 1.f,
                          0.f, none, &op->launches));
  // 2) P2[c][j][(i,s)] = sum_b Uy[j,b] P1[(b + ry*c)][(i,s)]   batch over c
  TTG_TRY(gemm<EPI_STORE>(st, ny, nx * S, ry, rz, Operand{Uy, 1, ny, 0},
                          Operand{P1, (int64_t)nx * S, 1, (int64_t)ry * nx * S}, P2,
                          (int64_t)nx * S, 1, (int64_t)ny * nx * S, 1.f, 0.f, none,
                          &op->launches));
  // 3) psi[l][(j,i,s)] = sum_c Uz[l,c] P2[c][(j,i,s)], fused: rho[i,j,l] += w_s psi^2
  //    column n = (j*nx + i)*S + s -> p = j*nx + i -> rho index i + nx*(j + ny*l) = p + nx*ny*l
  SqSum sq{rho, w, S, (int64_t)nx * ny, 1};
  TTG_TRY(gemm<EPI_SQSUM>(st, nz, ny * nx * S, rz, 1, Operand{Uz, 1, nz, 0},
                          Operand{P2, (int64_t)ny * nx * S, 1, 0}, nullptr, 0, 0, 0, 1.f, 0.f,
                          sq, &op->launches));
  const int64_t ng = (int64_t)nx * ny * nz;
  k_f2d<<<blocks_for(ng), 256, 0, st>>>(rho, stage, ng); TTG_COUNT();
  TTG_LAUNCHED(op);
  TTG_CUDA_TRY(cudaMemcpyAsync(rho_host, stage, ng * 8, cudaMemcpyDeviceToHost, st));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  return TTG_OK;
}

ttg_status ttg_hartree(int32_t K, const double* alpha, const double* omega, int32_t rx,
                       int32_t ry, int32_t rz, const double* G, int32_t nqx, int32_t nqy,
                       int32_t nqz, const double* xq, const double* yq, const double* zq,
                       const double* wqx, const double* wqy, const double* wqz,
                       const double* ux, const double* uy, const double* uz, int32_t nx,
                       int32_t ny, int32_t nz, const double* x, const double* y, const double* z,
                       double* v_host, float* kernel_ms) {
  if (K <= 0 || rx <= 0 || ry <= 0 || rz <= 0 || nx <= 0 || ny <= 0 || nz <= 0 || !alpha ||
      !omega || !G || !v_host)
    return TTG_BAD_ARG;
  int32_t smc, ma, mi;
  TTG_TRY(ttg_device_query(&smc, &ma, &mi));
  cudaStream_t st;
  TTG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamDefault));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
  } guard{st};
  Scratch sc;
  const int nq[3] = {nqx, nqy, nqz}, rr[3] = {rx, ry, rz}, ng[3] = {nx, ny, nz};
  const double* hq[3] = {xq, yq, zq};
  const double* hw[3] = {wqx, wqy, wqz};
  const double* hu[3] = {ux, uy, uz};
  const double* hx[3] = {x, y, z};
  double* d_alpha = sc.get<double>(K);
  double* d_omega = sc.get<double>(K);
  if (!d_alpha || !d_omega) return TTG_OOM;
  TTG_CUDA_TRY(cudaMemcpyAsync(d_alpha, alpha, K * 8, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(d_omega, omega, K * 8, cudaMemcpyHostToDevice, st));
  float* F[3];
  for (int d = 0; d < 3; ++d) {
    if (!hq[d] || !hw[d] || !hu[d] || !hx[d] || nq[d] <= 0) return TTG_BAD_ARG;
    double* dq = sc.get<double>(nq[d]);
    double* dw = sc.get<double>(nq[d]);
    double* du = sc.get<double>((int64_t)nq[d] * rr[d]);
    double* dx = sc.get<double>(ng[d]);
    F[d] = sc.get<float>((int64_t)K * ng[d] * rr[d]);
    if (!dq || !dw || !du || !dx || !F[d]) return TTG_OOM;
    TTG_CUDA_TRY(cudaMemcpyAsync(dq, hq[d], nq[d] * 8, cudaMemcpyHostToDevice, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(dw, hw[d], nq[d] * 8, cudaMemcpyHostToDevice, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(du, hu[d], (int64_t)nq[d] * rr[d] * 8, cudaMemcpyHostToDevice, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(dx, hx[d], ng[d] * 8, cudaMemcpyHostToDevice, st));
    // the z factor carries the term weight: B_big[(t,c), l] = w_t Fz_t[l, c]
    k_expansion_factor<<<dim3(1, ng[d], K), 128, nq[d] * 8, st>>>(
        d_alpha, K, dx, ng[d], dq, dw, nq[d], du, rr[d], F[d], d == 2 ? d_omega : nullptr); TTG_COUNT();
    if (cudaGetLastError() != cudaSuccess) return TTG_CUDA_ERR;
  }
  const int64_t ncore = (int64_t)rx * ry * rz;
  double* dG = sc.get<double>(ncore);
  float* Gf = sc.get<float>(ncore);
  float* P = sc.get<float>((int64_t)K * nx * ry * rz);        // [t][bc][i]
  float* Q = sc.get<float>((int64_t)K * rz * nx * ny);        // [(t,c)][(i,j)]
  const int64_t nout = (int64_t)nx * ny * nz;
  float* V = sc.get<float>(nout);
  double* Vd = sc.get<double>(nout);
  if (!dG || !Gf || !P || !Q || !V || !Vd) return TTG_OOM;
  TTG_CUDA_TRY(cudaMemcpyAsync(dG, G, ncore * 8, cudaMemcpyHostToDevice, st));
  k_d2f<<<blocks_for(ncore), 256, 0, st>>>(dG, Gf, ncore); TTG_COUNT();
  SqSum none{nullptr, nullptr, 1, 0, 0};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  // 1) P_t[i, bc] = sum_a Fx_t[i,a] G[a, bc]   (batch over t; A shared core)
  //    store P_t as [bc][i] (i fastest): element (m=i, n=bc) at i + nx*bc
  TTG_TRY(gemm<EPI_STORE>(st, nx, ry * rz, rx, K, Operand{F[0], rx, 1, (int64_t)nx * rx},
                          Operand{Gf, 1, rx, 0}, P, 1, nx, (int64_t)nx * ry * rz, 1.f, 0.f,
                          none, nullptr));
  // 2) Q_t[i, j, c] = sum_b P_t[i, b, c] Fy_t[j, b]   batch over (t, c)
  //    A(m=i, k=b) = P[t][b + ry*c][i] -> i + nx*(b + ry*c) + t*nx*ry*rz
  //    B(k=b, n=j) = Fy_t[j][b]  -> t*ny*ry + j*ry + b
  //    C(m=i, n=j) -> Q[(t*rz + c)][i + nx*j]
  //    one launch over z = t*rz + c: A offset nx*ry*z, B offset (z / rz)*ny*ry, C offset nx*ny*z
  TTG_TRY(gemm<EPI_STORE>(st, nx, ny, ry, K * rz, Operand{P, 1, nx, (int64_t)nx * ry, 1},
                          Operand{F[1], 1, ry, (int64_t)ny * ry, rz}, Q, 1, nx, (int64_t)nx * ny,
                          1.f, 0.f, none, nullptr));
  // 3) V[(i,j), l] = sum_{(t,c)} Q[(t,c)][(i,j)] * w_t Fz_t[l, c]   -- one launch, all K terms
  //    A(m=(i,j), k=(t,c)) at m + nx*ny*k;  B(k=(t,c), n=l) = Fz[t][l][c] -> t*nz*rz + l*rz + c
  //    the (t,c) -> t*nz*rz + c split is not a single stride, so gather B first
  float* Bz = sc.get<float>((int64_t)K * rz * nz);
  if (!Bz) return TTG_OOM;
  // Bz[(t*rz + c) + (K*rz)*l] = Fz[t][l][c]
  for (int t = 0; t < K; ++t)
    TTG_CUDA_TRY(cudaMemcpy2DAsync(Bz + (int64_t)t * rz, (size_t)K * rz * 4,
                                   F[2] + (int64_t)t * nz * rz, (size_t)rz * 4, (size_t)rz * 4, nz,
                                   cudaMemcpyDeviceToDevice, st));
  TTG_TRY(gemm<EPI_STORE>(st, nx * ny, nz, K * rz, 1, Operand{Q, 1, (int64_t)nx * ny, 0},
                          Operand{Bz, 1, (int64_t)K * rz, 0}, V, 1, (int64_t)nx * ny, 0, 1.f, 0.f,
                          none, nullptr));
  cudaEventRecord(e1, st);
  k_f2d<<<blocks_for(nout), 256, 0, st>>>(V, Vd, nout); TTG_COUNT();
  TTG_CUDA_TRY(cudaMemcpyAsync(v_host, Vd, nout * 8, cudaMemcpyDeviceToHost, st));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  if (kernel_ms) cudaEventElapsedTime(kernel_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return TTG_OK;
}

}  // extern "C"
