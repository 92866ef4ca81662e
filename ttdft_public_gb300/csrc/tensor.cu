// Tucker-mode contractions on the tensor cores: the density build
// (ProjectHamiltonianSparse::computeRhoOut, dft/ProjectHamiltonianSparse.cc:
// 911-1221, per-state ttm chain :1051-1074) and the Hartree kernel expansion
// (KSDFTPotential::computeHartreePotNew, dft/KSDFTPotential.cc:269-340; factor
// integrals :440-599; per-term ttm + daxpy :601-658).
//
// Both are chains of mode products, each one launch of the persistent
// tcgen05 contraction of tgemm.cu (FP32 operands cut into exact integer
// slices, no accumulation rounding, double-FP32 sums over groups).  The
// kernels that write an operand also record its largest |value| per group,
// which sets the contraction's slicing grid.
//
// Hartree: the dominant mode-3 product runs over all K expansion terms in one
// launch, V[(i,j), l] = sum_t sum_c Q_t[(i,j), c] (w_t Fz_t[l, c]), one
// group per term summed in double-FP32 by the epilogue, so V is written once
// (the reference updates it K times with a daxpy per term,
// KSDFTPotential.cc:641-654) and its accuracy does not degrade with K.
//
// Density: the last mode product squares, weights and sums over the states
// in its epilogue, rho[i,j,l] = sum_s 2 f_s psi_s[i,j,l]^2, so the per-state
// orbitals psi_s on the nodal grid are never written to HBM; states are
// processed in chunks so the intermediates stay within a fixed budget.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "ttg_internal.cuh"
#include "tgemm.cuh"

namespace ttg {
namespace {

int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 16);
}

int64_t rup(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

ttg_status grow(DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes) return TTG_OK;
  return b.alloc(bytes);
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

// the warp's largest |v| into *amax (FP32 bits compare as unsigned for v >= 0)
__device__ __forceinline__ void warp_max_abs(float* amax, float v) {
  const unsigned int m = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(v)));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(reinterpret_cast<unsigned int*>(amax), m);
}

// F_t[i, a] = scale_t sum_q wq[q] exp(-alpha_t (x_i - xq_q)^2) U[q, a] in
// FP64 on the CUDA cores (KSDFTPotential.cc:509-523), stored FP32 at
// out[t ost + i osi + a] for a < r and zero for r <= a < rpad; amax[t] gets
// the term's largest |F|.
__global__ void k_hfactor(const double* __restrict__ alpha, const double* __restrict__ x, int nx,
                          const double* __restrict__ xq, const double* __restrict__ wq, int nq,
                          const double* __restrict__ U, int r, int rpad, float* __restrict__ out,
                          int64_t ost, int64_t osi, const double* __restrict__ scale,
                          float* __restrict__ amax) {
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
  float* o = out + (int64_t)t * ost + (int64_t)i * osi;
  float vmax = 0.f;
  for (int a = threadIdx.x; a < rpad; a += blockDim.x) {
    double s = 0.0;
    if (a < r)
      for (int q = 0; q < nq; ++q) s += e[q] * U[q + (int64_t)a * nq];
    o[a] = (float)(sc * s);
    vmax = fmaxf(vmax, fabsf(o[a]));
  }
  warp_max_abs(amax + t, vmax);
}

// G (x fastest, rx * ry * rz) -> FP32 rows (b + ry c) of stride rxp
__global__ void k_core_rows(const double* __restrict__ G, int rx, int64_t rows, int rxp,
                            float* __restrict__ out, float* __restrict__ amax) {
  const int64_t n = rows * rx;
  float vmax = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = e / rx;
    const int a = (int)(e - row * rx);
    const float v = (float)G[e];
    out[row * rxp + a] = v;
    vmax = fmaxf(vmax, fabsf(v));
  }
  warp_max_abs(amax, vmax);
}

// FP64 column-major basis values (n x r) -> FP32 [i][a], row stride rp
__global__ void k_basis_rows(const double* __restrict__ U, int n, int r, int rp,
                             float* __restrict__ out, float* __restrict__ amax) {
  const int64_t total = (int64_t)n * r;
  float vmax = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / r), a = (int)(e - (int64_t)i * r);
    const float v = (float)U[i + (int64_t)a * n];
    out[(int64_t)i * rp + a] = v;
    vmax = fmaxf(vmax, fabsf(v));
  }
  warp_max_abs(amax, vmax);
}

// state s0 + blockIdx.y of the FP64 row-major block -> FP32 [s][(b, c)][a],
// row stride rxp; amax[s] gets the state's largest |value|
__global__ void k_block_chunk(const double* __restrict__ X, int64_t n, int64_t ld, int s0, int rx,
                              int rxp, float* __restrict__ out, float* __restrict__ amax) {
  const int64_t rows = n / rx;
  const int s = blockIdx.y;
  float vmax = 0.f;
  for (int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; I < n;
       I += (int64_t)gridDim.x * blockDim.x) {
    const int64_t bc = I / rx;
    const int a = (int)(I - bc * rx);
    const float v = (float)X[I * ld + s0 + s];
    out[((int64_t)s * rows + bc) * rxp + a] = v;
    vmax = fmaxf(vmax, fabsf(v));
  }
  warp_max_abs(amax + s, vmax);
}

// Device inputs of one Hartree evaluation (all FP64, device pointers).
struct HartreeIn {
  int K;
  const double *alpha, *omega;
  int r[3];
  const double* G;              // r0 r1 r2, x fastest
  int nq[3];
  const double *xq[3], *wq[3];
  const double* U[3];           // nq_d x r_d column-major
  int n[3];
  const double* x[3];           // target points
};

ttg_status ensure_err(HartreeWork& w, cudaStream_t st) {
  if (w.err.p) return TTG_OK;
  TTG_TRY(w.err.alloc(sizeof(int)));
  TTG_CUDA_TRY(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
  return TTG_OK;
}

// V (FP64, x fastest on the target grid) = sum_t omega_t G x1 Fx_t x2 Fy_t x3 Fz_t:
// three tensor-core contractions (tgemm.cu), the last one summing the K terms
// in double-FP32, one group per term.
ttg_status hartree_tc(cudaStream_t st, HartreeWork& w, const HartreeIn& in, double* V,
                      cudaEvent_t e0, cudaEvent_t e1) {
  const int K = in.K, rx = in.r[0], ry = in.r[1], rz = in.r[2];
  const int nx = in.n[0], ny = in.n[1], nz = in.n[2];
  const int64_t rxp = rup(rx, 4), ryp = rup(ry, 4), ktt = rup(rz, 16), kt = (int64_t)K * ktt;
  if (ktt > 192 || rx > 192 || ry > 192) return TTG_BAD_ARG;
  TTG_TRY(grow(w.F[0], (size_t)K * nx * rxp * 4));
  TTG_TRY(grow(w.F[1], (size_t)K * ny * ryp * 4));
  TTG_TRY(grow(w.F[2], (size_t)nz * kt * 4));
  TTG_TRY(grow(w.gf, (size_t)ry * rz * rxp * 4));
  TTG_TRY(grow(w.p2, (size_t)K * nx * rz * ryp * 4));
  const int64_t qrows = (int64_t)nx * ny;
  if (w.q.bytes < (size_t)(qrows * kt * 4) || w.q_layout[0] != qrows || w.q_layout[1] != K ||
      w.q_layout[2] != ktt) {
    // the padding columns (t, c >= rz) of Q are never written: zero them once
    TTG_TRY(grow(w.q, (size_t)(qrows * kt * 4)));
    TTG_CUDA_TRY(cudaMemsetAsync(w.q.p, 0, (size_t)(qrows * kt * 4), st));
    w.q_layout[0] = qrows;
    w.q_layout[1] = K;
    w.q_layout[2] = ktt;
  }
  TTG_TRY(ensure_err(w, st));
  // group maxima of the operands: [G][Fx: K][Fy: K][Fz: K][P: K][Q: K]
  TTG_TRY(grow(w.amax, (size_t)(1 + 5 * K) * 4));
  TTG_CUDA_TRY(cudaMemsetAsync(w.amax.p, 0, (size_t)(1 + 5 * K) * 4, st));
  float* am = w.amax.as<float>();
  float* am_g = am;
  float* am_f[3] = {am + 1, am + 1 + K, am + 1 + 2 * K};
  float* am_p = am + 1 + 3 * K;
  float* am_q = am + 1 + 4 * K;
  // expansion factors (FP64 integrals, FP32 storage); the z factor carries
  // the term weight and is laid out [l][(t, c)] with zero padding per term
  const int64_t ost[3] = {(int64_t)nx * rxp, (int64_t)ny * ryp, ktt};
  const int64_t osi[3] = {rxp, ryp, kt};
  const int rpad[3] = {(int)rxp, (int)ryp, (int)ktt};
  for (int d = 0; d < 3; ++d) {
    k_hfactor<<<dim3(1, in.n[d], K), 128, in.nq[d] * 8, st>>>(
        in.alpha, in.x[d], in.n[d], in.xq[d], in.wq[d], in.nq[d], in.U[d], in.r[d], rpad[d],
        w.F[d].as<float>(), ost[d], osi[d], d == 2 ? in.omega : nullptr, am_f[d]); TTG_COUNT();
    TTG_CUDA_TRY(cudaGetLastError());
  }
  k_core_rows<<<blocks_for((int64_t)rx * ry * rz), 256, 0, st>>>(
      in.G, rx, (int64_t)ry * rz, (int)rxp, w.gf.as<float>(), am_g); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  if (e0) TTG_CUDA_TRY(cudaEventRecord(e0, st));
  int* err = w.err.as<int>();
  // 1) P_t[(i, c)][b] = sum_a G[(b, c)][a] Fx_t[i][a]      rows (b, c) x cols i, batch t
  TOperand A1{w.gf.as<float>(), (int64_t)ry * rz, rx, rxp, 0, 0, am_g};
  TOperand B1{w.F[0].as<float>(), nx, rx, rxp, K, (int64_t)nx * rxp, am_f[0]};
  TOut o1{w.p2.p, ry, 1, ryp, (int64_t)rz * ryp, (int64_t)nx * rz * ryp};
  o1.omax = am_p;
  o1.limit = (int64_t)K * nx * rz * ryp;
  TTG_TRY(tgemm(st, TG_STORE_F32, A1, B1, K, 1, (int)((rx + 15) / 16), o1, err));
  // 2) Q[(i + nx j)][(t, c)] = sum_b P_t[(i, c)][b] Fy_t[j][b]   rows (i, c) x cols j, batch t
  TOperand A2{w.p2.as<float>(), (int64_t)nx * rz, ry, ryp, K, (int64_t)nx * rz * ryp, am_p};
  TOperand B2{w.F[1].as<float>(), ny, ry, ryp, K, (int64_t)ny * ryp, am_f[1]};
  TOut o2{w.q.p, rz, 1, kt, (int64_t)nx * kt, ktt};
  o2.omax = am_q;
  o2.limit = qrows * kt;
  TTG_TRY(tgemm(st, TG_STORE_F32, A2, B2, K, 1, (int)((ry + 15) / 16), o2, err));
  // 3) V[(i, j), l] = sum_t sum_c Q[(i, j)][(t, c)] w_t Fz_t[l][c], one group per term
  TOperand A3{w.q.as<float>(), qrows, kt, kt, 0, 0, am_q};
  TOperand B3{w.F[2].as<float>(), nz, kt, kt, 0, 0, am_f[2]};
  TOut o3{V, qrows + 1, 1, 0, qrows, 0};
  o3.limit = qrows * nz;
  TTG_TRY(tgemm(st, TG_SUM_F64, A3, B3, 1, K, (int)(ktt / 16), o3, err));
  if (e1) TTG_CUDA_TRY(cudaEventRecord(e1, st));
  return TTG_OK;
}

ttg_status hartree_check(HartreeWork& w, cudaStream_t st) {
  if (!w.err.p) return TTG_OK;
  int e = 0;
  TTG_CUDA_TRY(cudaMemcpyAsync(&e, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  if (e) {
    TTG_CUDA_TRY(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
    if (e == 2) {
      fprintf(stderr, "ttg: a tensor-core contraction skipped stores outside its output\n");
      return TTG_BAD_ARG;
    }
    if (e == 3) {
      fprintf(stderr, "ttg: a tensor-core contraction found a copy barrier out of phase\n");
      return TTG_CUDA_ERR;
    }
    return TTG_TIMEOUT;
  }
  return TTG_OK;
}

// rho[i, j, l] (+)= sum_s 2 f_s psi_s[i, j, l]^2, psi_s = c_s x1 Ux x2 Uy x3 Uz,
// in chunks of states: two batched tensor-core mode products and a third one
// whose epilogue squares, weights and sums over the chunk's states in
// double-FP32 (tgemm.cu).
ttg_status density_tc(ttg_op* op, const ttg_block* X, const double* occ, int rx, int ry, int rz,
                      int nx, int ny, int nz, const double* ux, const double* uy,
                      const double* uz, double* rho, bool accumulate) {
  DensityWork& D = op->dw;
  cudaStream_t st = op->stream;
  const int k = X->k;
  const int64_t rxp = rup(rx, 4), ryp = rup(ry, 4), rzp = rup(rz, 4);
  if (rx > 192 || ry > 192 || rz > 192) return TTG_BAD_ARG;
  const int rr[3] = {rx, ry, rz}, nn[3] = {nx, ny, nz};
  const int64_t rp[3] = {rxp, ryp, rzp};
  const double* U[3] = {ux, uy, uz};
  // group maxima: [Ux][Uy][Uz][X_s: S][P1_s: S][P2_s: S]
  TTG_TRY(grow(D.amax, (size_t)(3 + 3 * (int64_t)k) * 4));
  float* dm = D.amax.as<float>();
  TTG_CUDA_TRY(cudaMemsetAsync(dm, 0, 3 * 4, st));
  for (int d = 0; d < 3; ++d) {
    TTG_TRY(grow(D.uf[d], (size_t)nn[d] * rp[d] * 4));
    k_basis_rows<<<blocks_for((int64_t)nn[d] * rr[d]), 256, 0, st>>>(
        U[d], nn[d], rr[d], (int)rp[d], D.uf[d].as<float>(), dm + d); TTG_COUNT();
    TTG_LAUNCHED(op);
  }
  TTG_TRY(ensure_err(op->hw, st));
  // states per chunk: the three intermediates within a fixed budget
  const int64_t per_state = ((int64_t)ry * rz * rxp + (int64_t)rz * nx * ryp +
                             (int64_t)ny * nx * rzp) * 4;
  const char* env = getenv("TTG_DENSITY_CHUNK_BYTES");
  const int64_t budget = env ? std::max<int64_t>(atoll(env), 1) : ((int64_t)3 << 30);
  const int S = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)k, budget / per_state, 65535}));
  TTG_TRY(grow(D.xt, (size_t)S * ry * rz * rxp * 4));
  TTG_TRY(grow(D.p1, (size_t)S * rz * nx * ryp * 4));
  TTG_TRY(grow(D.p2, (size_t)S * ny * nx * rzp * 4));
  TTG_TRY(grow(D.w, (size_t)k * 4));
  std::vector<float> wh(k);
  for (int s = 0; s < k; ++s) wh[s] = (float)(2.0 * occ[s]);
  TTG_CUDA_TRY(cudaMemcpyAsync(D.w.p, wh.data(), (size_t)k * 4, cudaMemcpyHostToDevice, st));
  int* err = op->hw.err.as<int>();
  for (int s0 = 0; s0 < k; s0 += S) {
    const int sc = std::min(S, k - s0);
    float* am_x = dm + 3;
    float* am_1 = am_x + S;
    float* am_2 = am_1 + S;
    TTG_CUDA_TRY(cudaMemsetAsync(am_x, 0, (size_t)3 * S * 4, st));
    const int gx = (int)std::min<int64_t>((op->n + 255) / 256, 64);
    k_block_chunk<<<dim3(gx, sc), 256, 0, st>>>(X->x.as<double>(), op->n, op->ld, s0, rx,
                                                (int)rxp, D.xt.as<float>(), am_x); TTG_COUNT();
    TTG_LAUNCHED(op);
    // 1) P1[s][c][i][b] = sum_a X_s[(b, c)][a] Ux[i][a]       rows (b, c), cols i, batch s
    TOperand A1{D.xt.as<float>(), (int64_t)ry * rz, rx, rxp, sc, (int64_t)ry * rz * rxp, am_x};
    TOperand B1{D.uf[0].as<float>(), nx, rx, rxp, 0, 0, dm};
    TOut o1{D.p1.p, ry, 1, (int64_t)nx * ryp, ryp, (int64_t)rz * nx * ryp};
    o1.omax = am_1;
    o1.limit = (int64_t)sc * rz * nx * ryp;
    TTG_TRY(tgemm(st, TG_STORE_F32, A1, B1, sc, 1, (rx + 15) / 16, o1, err));
    // 2) P2[s][j][i][c] = sum_b P1[s][(c, i)][b] Uy[j][b]       rows (c, i), cols j, batch s
    TOperand A2{D.p1.as<float>(), (int64_t)rz * nx, ry, ryp, sc, (int64_t)rz * nx * ryp, am_1};
    TOperand B2{D.uf[1].as<float>(), ny, ry, ryp, 0, 0, dm + 1};
    TOut o2{D.p2.p, nx, rzp, 1, (int64_t)nx * rzp, (int64_t)ny * nx * rzp};
    o2.omax = am_2;
    o2.limit = (int64_t)sc * ny * nx * rzp;
    TTG_TRY(tgemm(st, TG_STORE_F32, A2, B2, sc, 1, (ry + 15) / 16, o2, err));
    // 3) rho[(i, j), l] (+)= sum_s w_s (sum_c P2[s][(j, i)][c] Uz[l][c])^2
    TOperand A3{D.p2.as<float>(), (int64_t)nx * ny, rz, rzp, sc, (int64_t)ny * nx * rzp, am_2};
    TOperand B3{D.uf[2].as<float>(), nz, rz, rzp, 0, 0, dm + 2};
    TOut o3{rho, (int64_t)nx * ny + 1, 1, 0, (int64_t)nx * ny, 0, D.w.as<float>() + s0,
            (accumulate || s0 > 0) ? 1 : 0};
    o3.limit = (int64_t)nx * ny * nz;
    TTG_TRY(tgemm(st, TG_SQSUM_F64, A3, B3, 1, sc, (rz + 15) / 16, o3, err));
    op->launches += 3;
  }
  return TTG_OK;
}

}  // namespace

ttg_status hartree_error(ttg_op* op) { return hartree_check(op->hw, op->stream); }

}  // namespace ttg

using namespace ttg;

extern "C" {

ttg_status ttg_density_device(ttg_op* op, const ttg_block* X, const double* occ_host,
                              const int32_t* ranks, const int32_t* n, const double* ux_dev,
                              const double* uy_dev, const double* uz_dev, double* rho_dev,
                              int32_t accumulate) {
  if (!op || !X || X->op != op || !occ_host || !ranks || !n || !ux_dev || !uy_dev || !uz_dev ||
      !rho_dev)
    return TTG_BAD_ARG;
  const int rx = ranks[0], ry = ranks[1], rz = ranks[2];
  const int nx = n[0], ny = n[1], nz = n[2];
  if (rx <= 0 || ry <= 0 || rz <= 0 || nx <= 0 || ny <= 0 || nz <= 0 ||
      (int64_t)rx * ry * rz != op->n)
    return TTG_BAD_ARG;
  TTG_TRY(kt_begin(op, TTG_KT_DENSITY));
  TTG_TRY(density_tc(op, X, occ_host, rx, ry, rz, nx, ny, nz, ux_dev, uy_dev, uz_dev, rho_dev,
                     accumulate != 0));
  TTG_TRY(kt_end(op));
  return TTG_OK;
}

ttg_status ttg_density(ttg_op* op, const ttg_block* X, const double* occ_host, int32_t rx,
                       int32_t ry, int32_t rz, int32_t nx, int32_t ny, int32_t nz,
                       const double* ux, const double* uy, const double* uz, double* rho_host) {
  if (!op || !X || X->op != op || !occ_host || !ux || !uy || !uz || !rho_host) return TTG_BAD_ARG;
  if ((int64_t)rx * ry * rz != op->n || nx <= 0 || ny <= 0 || nz <= 0) return TTG_BAD_ARG;
  cudaStream_t st = op->stream;
  Scratch sc;
  const int64_t ng = (int64_t)nx * ny * nz;
  const int nn[3] = {nx, ny, nz}, rr[3] = {rx, ry, rz};
  const double* hu[3] = {ux, uy, uz};
  double* du[3];
  for (int d = 0; d < 3; ++d) {
    du[d] = sc.get<double>((int64_t)nn[d] * rr[d]);
    if (!du[d]) return TTG_OOM;
    TTG_CUDA_TRY(cudaMemcpyAsync(du[d], hu[d], (size_t)nn[d] * rr[d] * 8, cudaMemcpyHostToDevice, st));
  }
  double* rho = sc.get<double>(ng);
  if (!rho) return TTG_OOM;
  TTG_TRY(density_tc(op, X, occ_host, rx, ry, rz, nx, ny, nz, du[0], du[1], du[2], rho, false));
  TTG_TRY(hartree_check(op->hw, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(rho_host, rho, ng * 8, cudaMemcpyDeviceToHost, st));
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
  struct Guard {
    cudaStream_t s;
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Guard() {
      cudaStreamSynchronize(s);
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
      cudaStreamDestroy(s);
    }
  } guard{st};
  TTG_CUDA_TRY(cudaEventCreate(&guard.e[0]));
  TTG_CUDA_TRY(cudaEventCreate(&guard.e[1]));
  HartreeWork w;
  Scratch sc;
  const int nq[3] = {nqx, nqy, nqz}, rr[3] = {rx, ry, rz}, ng[3] = {nx, ny, nz};
  const double* hq[3] = {xq, yq, zq};
  const double* hw[3] = {wqx, wqy, wqz};
  const double* hu[3] = {ux, uy, uz};
  const double* hx[3] = {x, y, z};
  HartreeIn in;
  in.K = K;
  double* d_alpha = sc.get<double>(K);
  double* d_omega = sc.get<double>(K);
  double* dG = sc.get<double>((int64_t)rx * ry * rz);
  const int64_t nout = (int64_t)nx * ny * nz;
  double* V = sc.get<double>(nout);
  if (!d_alpha || !d_omega || !dG || !V) return TTG_OOM;
  TTG_CUDA_TRY(cudaMemcpyAsync(d_alpha, alpha, K * 8, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(d_omega, omega, K * 8, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(dG, G, (size_t)rx * ry * rz * 8, cudaMemcpyHostToDevice, st));
  in.alpha = d_alpha;
  in.omega = d_omega;
  in.G = dG;
  for (int d = 0; d < 3; ++d) {
    if (!hq[d] || !hw[d] || !hu[d] || !hx[d] || nq[d] <= 0) return TTG_BAD_ARG;
    double* dq = sc.get<double>(nq[d]);
    double* dw = sc.get<double>(nq[d]);
    double* du = sc.get<double>((int64_t)nq[d] * rr[d]);
    double* dx = sc.get<double>(ng[d]);
    if (!dq || !dw || !du || !dx) return TTG_OOM;
    TTG_CUDA_TRY(cudaMemcpyAsync(dq, hq[d], nq[d] * 8, cudaMemcpyHostToDevice, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(dw, hw[d], nq[d] * 8, cudaMemcpyHostToDevice, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(du, hu[d], (int64_t)nq[d] * rr[d] * 8, cudaMemcpyHostToDevice, st));
    TTG_CUDA_TRY(cudaMemcpyAsync(dx, hx[d], ng[d] * 8, cudaMemcpyHostToDevice, st));
    in.r[d] = rr[d];
    in.nq[d] = nq[d];
    in.xq[d] = dq;
    in.wq[d] = dw;
    in.U[d] = du;
    in.n[d] = ng[d];
    in.x[d] = dx;
  }
  TTG_TRY(hartree_tc(st, w, in, V, guard.e[0], guard.e[1]));
  TTG_TRY(hartree_check(w, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(v_host, V, nout * 8, cudaMemcpyDeviceToHost, st));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  if (kernel_ms) TTG_CUDA_TRY(cudaEventElapsedTime(kernel_ms, guard.e[0], guard.e[1]));
  return TTG_OK;
}

ttg_status ttg_hartree_device(ttg_op* op, int32_t K, const double* alpha_dev,
                              const double* omega_dev, const int32_t* ranks, const double* g_dev,
                              const int32_t* nq, const double* const* xq_dev,
                              const double* const* wq_dev, const double* const* u_dev,
                              const int32_t* n, const double* const* x_dev, double* v_dev) {
  if (!op || K <= 0 || !alpha_dev || !omega_dev || !ranks || !g_dev || !nq || !xq_dev ||
      !wq_dev || !u_dev || !n || !x_dev || !v_dev)
    return TTG_BAD_ARG;
  HartreeIn in;
  in.K = K;
  in.alpha = alpha_dev;
  in.omega = omega_dev;
  in.G = g_dev;
  for (int d = 0; d < 3; ++d) {
    if (ranks[d] <= 0 || nq[d] <= 0 || n[d] <= 0 || !xq_dev[d] || !wq_dev[d] || !u_dev[d] ||
        !x_dev[d])
      return TTG_BAD_ARG;
    in.r[d] = ranks[d];
    in.nq[d] = nq[d];
    in.xq[d] = xq_dev[d];
    in.wq[d] = wq_dev[d];
    in.U[d] = u_dev[d];
    in.n[d] = n[d];
    in.x[d] = x_dev[d];
  }
  TTG_TRY(kt_begin(op, TTG_KT_HARTREE));
  TTG_TRY(hartree_tc(op->stream, op->hw, in, v_dev, nullptr, nullptr));
  TTG_TRY(kt_end(op));
  op->launches += 7;
  return TTG_OK;
}

}  // extern "C"
