// Learned initial density: per-atom descriptors and a small multilayer
// perceptron trained and evaluated by the kernels in this file (FP32).
//
// Descriptor of atom a (pairwise Gaussian radial features, cosine cutoff):
//   D_a[m] = sum_{b != a} exp(-eta (r_ab - mu_m)^2) fc(r_ab),
//   fc(r) = (cos(pi r / rc) + 1) / 2 for r < rc, else 0.
// Network: layers l = 0..L-1, Z_l = H_l W_l + b_l (W_l: in x out, row-major),
// H_{l+1} = tanh(Z_l) for hidden layers, the last layer linear.  Loss:
// mean over samples of sum_j (Y_j - T_j)^2.  Backward pass by the chain rule,
// Adam (Kingma & Ba, ICLR 2015) with decoupled weight decay on the weights.
// The reference has no counterpart (its initial guess is the superposition
// of atomic densities, dft/InitialGuess.cc:573-681, kept as the fallback).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ttg_internal.cuh"

struct ttg_mlp {
  int n_layers = 0;
  std::vector<int> sizes;                 // n_layers + 1
  std::vector<int64_t> w_off, b_off;      // offsets into the parameter vector
  int64_t n_params = 0;
  ttg::DevBuf params, grads, m1, m2;      // FP32, n_params each
  ttg::DevBuf acts;                       // activations of a batch (grow-only)
  ttg::DevBuf dbuf;                       // deltas of a batch (grow-only)
  ttg::DevBuf tbuf, loss;                 // batch targets / loss partials
  int64_t step = 0;
  cudaStream_t stream = nullptr;
};

namespace ttg {
namespace {

constexpr int kT = 16;   // tile of the small GEMMs

// C (M x N) = A (M x K) B (K x N) [+ bias] with optional transposes, row-major.
// ta: A given as K x M; tb: B given as N x K.  act 1: C = tanh(C).
__global__ void k_mlp_gemm(const float* __restrict__ A, const float* __restrict__ B,
                           const float* __restrict__ bias, float* __restrict__ C, int M, int N,
                           int K, int ta, int tb, int act, int accumulate) {
  __shared__ float sA[kT][kT + 1];
  __shared__ float sB[kT][kT + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * kT + ty, col = blockIdx.x * kT + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += kT) {
    const int ka = k0 + tx, kb = k0 + ty;
    float a = 0.f, b = 0.f;
    if (row < M && ka < K) a = ta ? A[(int64_t)ka * M + row] : A[(int64_t)row * K + ka];
    if (col < N && kb < K) b = tb ? B[(int64_t)col * K + kb] : B[(int64_t)kb * N + col];
    sA[ty][tx] = a;
    sB[ty][tx] = b;
    __syncthreads();
#pragma unroll
    for (int t = 0; t < kT; ++t) acc = fmaf(sA[ty][t], sB[t][tx], acc);
    __syncthreads();
  }
  if (row < M && col < N) {
    if (bias) acc += bias[col];
    if (act) acc = tanhf(acc);
    float* c = C + (int64_t)row * N + col;
    *c = accumulate ? *c + acc : acc;
  }
}

// dZ = dH * (1 - H^2) for a tanh layer (H = tanh(Z)), in place on dH.
__global__ void k_tanh_back(float* __restrict__ d, const float* __restrict__ h, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float y = h[i];
    d[i] *= 1.f - y * y;
  }
}

// Output delta of the mean squared error and the per-block loss:
// d = 2 (Y - T) / B, part[block] = sum (Y - T)^2.
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, int64_t n,
                      float inv_b, float* __restrict__ d, float* __restrict__ part) {
  __shared__ float red[32];
  float s = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float r = y[i] - t[i];
    d[i] = 2.f * r * inv_b;
    s += r * r;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    part[blockIdx.x] = tot;
  }
}

// db[j] = sum_i dZ[i][j]  (B x N), fixed order per column.
__global__ void k_colsum(const float* __restrict__ d, int B, int N, float* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0.f;
  for (int i = 0; i < B; ++i) s += d[(int64_t)i * N + j];
  out[j] = s;
}

// Adam with bias correction; weight decay (decoupled) only where decay != 0.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, float wd, const unsigned char* __restrict__ decay) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / c1, vh = vi / c2;
    float upd = mh / (sqrtf(vh) + eps);
    if (decay && decay[i]) upd += wd * p[i];
    p[i] -= lr * upd;
  }
}

__global__ void k_descriptors(const double* __restrict__ pos, int natoms, int nf, double mu0,
                              double dmu, double eta, double rc, float* __restrict__ out) {
  const int a = blockIdx.x;
  const double pi = 3.14159265358979323846;
  for (int m = threadIdx.x; m < nf; m += blockDim.x) {
    const double mu = mu0 + dmu * m;
    double s = 0.0;
    for (int b = 0; b < natoms; ++b) {
      if (b == a) continue;
      const double dx = pos[3 * a] - pos[3 * b], dy = pos[3 * a + 1] - pos[3 * b + 1],
                   dz = pos[3 * a + 2] - pos[3 * b + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r >= rc) continue;
      const double fc = 0.5 * (cos(pi * r / rc) + 1.0);
      s += exp(-eta * (r - mu) * (r - mu)) * fc;
    }
    out[(int64_t)a * nf + m] = (float)s;
  }
}

int grid1(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 8); }

void gemm(cudaStream_t st, const float* A, const float* B, const float* bias, float* C, int M,
          int N, int K, bool ta, bool tb, bool act, bool acc) {
  dim3 blk(kT, kT), grd((N + kT - 1) / kT, (M + kT - 1) / kT);
  k_mlp_gemm<<<grd, blk, 0, st>>>(A, B, bias, C, M, N, K, ta, tb, act, acc); TTG_COUNT();
}

int64_t act_size(const ttg_mlp* m, int B) {
  int64_t s = 0;
  for (int l = 0; l <= m->n_layers; ++l) s += (int64_t)B * m->sizes[l];
  return s;
}

ttg_status ensure_batch(ttg_mlp* m, int B) {
  const size_t need = (size_t)act_size(m, B) * 4;
  if (m->acts.bytes < need) TTG_TRY(m->acts.alloc(need));
  if (m->dbuf.bytes < need) TTG_TRY(m->dbuf.alloc(need));
  const size_t nout = (size_t)B * m->sizes[m->n_layers] * 4;
  if (m->tbuf.bytes < nout) TTG_TRY(m->tbuf.alloc(nout));
  if (m->loss.bytes < 152 * 8 * 4) TTG_TRY(m->loss.alloc(152 * 8 * 4));
  return TTG_OK;
}

// Activations (or deltas) of layer l for a batch of B, inside `base`.
float* act_ptr(ttg_mlp* m, int B, int l, float* base) {
  int64_t off = 0;
  for (int i = 0; i < l; ++i) off += (int64_t)B * m->sizes[i];
  return base + off;
}

void forward(ttg_mlp* m, int B) {
  float* P = m->params.as<float>();
  float* H = m->acts.as<float>();
  for (int l = 0; l < m->n_layers; ++l) {
    const bool last = (l == m->n_layers - 1);
    gemm(m->stream, act_ptr(m, B, l, H), P + m->w_off[l], P + m->b_off[l],
         act_ptr(m, B, l + 1, H), B, m->sizes[l + 1], m->sizes[l], false, false, !last, false);
  }
}

// Loss and parameter gradients of the batch whose inputs are the first
// activations and whose targets are in tbuf (forward first).
float backward(ttg_mlp* m, int B) {
  cudaStream_t st = m->stream;
  float* P = m->params.as<float>();
  float* G = m->grads.as<float>();
  float* H = m->acts.as<float>();
  float* D = m->dbuf.as<float>();
  const int L = m->n_layers;
  const int64_t nout = (int64_t)B * m->sizes[L];
  const int nb = grid1(nout);
  k_mse<<<nb, 256, 0, st>>>(act_ptr(m, B, L, H), m->tbuf.as<float>(), nout, 1.f / B,
                            act_ptr(m, B, L, D), m->loss.as<float>()); TTG_COUNT();
  for (int l = L - 1; l >= 0; --l) {
    float* dZ = act_ptr(m, B, l + 1, D);
    if (l != L - 1) {
      const int64_t n = (int64_t)B * m->sizes[l + 1];
      k_tanh_back<<<grid1(n), 256, 0, st>>>(dZ, act_ptr(m, B, l + 1, H), n); TTG_COUNT();
    }
    // dW = H_l^T dZ (in x out), db = colsum(dZ), dH_l = dZ W^T
    gemm(st, act_ptr(m, B, l, H), dZ, nullptr, G + m->w_off[l], m->sizes[l], m->sizes[l + 1], B,
         true, false, false, false);
    k_colsum<<<(m->sizes[l + 1] + 127) / 128, 128, 0, st>>>(dZ, B, m->sizes[l + 1],
                                                           G + m->b_off[l]); TTG_COUNT();
    if (l > 0)
      gemm(st, dZ, P + m->w_off[l], nullptr, act_ptr(m, B, l, D), B, m->sizes[l], m->sizes[l + 1],
           false, true, false, false);
  }
  std::vector<float> part(nb);
  cudaMemcpyAsync(part.data(), m->loss.p, nb * 4, cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += part[i];
  return (float)(s / B);
}

}  // namespace
}  // namespace ttg

extern "C" {

ttg_status ttg_mlp_create(int32_t n_layers, const int32_t* sizes, ttg_mlp** out) {
  if (!sizes || !out || n_layers < 1 || n_layers > 16) return TTG_BAD_ARG;
  auto* m = new ttg_mlp();
  m->n_layers = n_layers;
  for (int l = 0; l <= n_layers; ++l) {
    if (sizes[l] <= 0 || sizes[l] > 4096) {
      delete m;
      return TTG_BAD_ARG;
    }
    m->sizes.push_back(sizes[l]);
  }
  int64_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    m->w_off.push_back(off);
    off += (int64_t)sizes[l] * sizes[l + 1];
    m->b_off.push_back(off);
    off += sizes[l + 1];
  }
  m->n_params = off;
  ttg_status s;
  if ((s = m->params.alloc(off * 4)) != TTG_OK || (s = m->grads.alloc(off * 4)) != TTG_OK ||
      (s = m->m1.alloc(off * 4)) != TTG_OK || (s = m->m2.alloc(off * 4)) != TTG_OK) {
    delete m;
    return s;
  }
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamDefault) != cudaSuccess) {
    delete m;
    return TTG_CUDA_ERR;
  }
  cudaMemsetAsync(m->params.p, 0, off * 4, m->stream);
  cudaMemsetAsync(m->m1.p, 0, off * 4, m->stream);
  cudaMemsetAsync(m->m2.p, 0, off * 4, m->stream);
  *out = m;
  return TTG_OK;
}

void ttg_mlp_destroy(ttg_mlp* m) {
  if (!m) return;
  if (m->stream) {
    cudaStreamSynchronize(m->stream);
    cudaStreamDestroy(m->stream);
  }
  delete m;
}

int64_t ttg_mlp_num_params(const ttg_mlp* m) { return m ? m->n_params : -1; }

ttg_status ttg_mlp_set_params(ttg_mlp* m, const float* p) {
  if (!m || !p) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaMemcpyAsync(m->params.p, p, m->n_params * 4, cudaMemcpyHostToDevice, m->stream));
  TTG_CUDA_TRY(cudaMemsetAsync(m->m1.p, 0, m->n_params * 4, m->stream));
  TTG_CUDA_TRY(cudaMemsetAsync(m->m2.p, 0, m->n_params * 4, m->stream));
  m->step = 0;
  TTG_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return TTG_OK;
}

ttg_status ttg_mlp_get_params(ttg_mlp* m, float* p) {
  if (!m || !p) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaMemcpyAsync(p, m->params.p, m->n_params * 4, cudaMemcpyDeviceToHost, m->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return TTG_OK;
}

ttg_status ttg_mlp_forward(ttg_mlp* m, const float* x, int32_t n, float* y) {
  if (!m || !x || !y || n <= 0) return TTG_BAD_ARG;
  TTG_TRY(ttg::ensure_batch(m, n));
  float* H = m->acts.as<float>();
  TTG_CUDA_TRY(cudaMemcpyAsync(H, x, (size_t)n * m->sizes[0] * 4, cudaMemcpyHostToDevice,
                               m->stream));
  ttg::forward(m, n);
  TTG_CUDA_TRY(cudaGetLastError());
  TTG_CUDA_TRY(cudaMemcpyAsync(y, ttg::act_ptr(m, n, m->n_layers, H),
                               (size_t)n * m->sizes[m->n_layers] * 4, cudaMemcpyDeviceToHost,
                               m->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return TTG_OK;
}

ttg_status ttg_mlp_gradients(ttg_mlp* m, const float* x, const float* t, int32_t n, float* grad,
                             float* loss) {
  if (!m || !x || !t || !grad || !loss || n <= 0) return TTG_BAD_ARG;
  TTG_TRY(ttg::ensure_batch(m, n));
  float* H = m->acts.as<float>();
  TTG_CUDA_TRY(cudaMemcpyAsync(H, x, (size_t)n * m->sizes[0] * 4, cudaMemcpyHostToDevice,
                               m->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(m->tbuf.p, t, (size_t)n * m->sizes[m->n_layers] * 4,
                               cudaMemcpyHostToDevice, m->stream));
  ttg::forward(m, n);
  *loss = ttg::backward(m, n);
  TTG_CUDA_TRY(cudaGetLastError());
  TTG_CUDA_TRY(cudaMemcpyAsync(grad, m->grads.p, m->n_params * 4, cudaMemcpyDeviceToHost,
                               m->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return TTG_OK;
}

ttg_status ttg_mlp_train(ttg_mlp* m, const float* x, const float* t, int32_t n, int32_t epochs,
                         int32_t batch, float lr, float weight_decay, uint64_t seed,
                         float* loss_per_epoch) {
  if (!m || !x || !t || n <= 0 || epochs <= 0 || batch <= 0) return TTG_BAD_ARG;
  const int B = std::min<int>(batch, n);
  const int nin = m->sizes[0], nout = m->sizes[m->n_layers];
  TTG_TRY(ttg::ensure_batch(m, B));
  ttg::DevBuf dx, dt, mask;
  TTG_TRY(dx.alloc((size_t)n * nin * 4));
  TTG_TRY(dt.alloc((size_t)n * nout * 4));
  TTG_TRY(mask.alloc(m->n_params));
  std::vector<unsigned char> hm(m->n_params, 0);
  for (int l = 0; l < m->n_layers; ++l)
    std::fill(hm.begin() + m->w_off[l], hm.begin() + m->b_off[l], 1);
  TTG_CUDA_TRY(cudaMemcpyAsync(mask.p, hm.data(), hm.size(), cudaMemcpyHostToDevice, m->stream));
  // samples reshuffled every epoch on the host and copied contiguously, so
  // that every batch is a contiguous slice
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  std::vector<float> xs((size_t)n * nin), ts((size_t)n * nout);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  float* H = m->acts.as<float>();
  for (int ep = 0; ep < epochs; ++ep) {
    for (int i = n - 1; i > 0; --i) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      const int j = (int)((st >> 33) % (uint64_t)(i + 1));
      std::swap(perm[i], perm[j]);
    }
    for (int i = 0; i < n; ++i) {
      std::memcpy(&xs[(size_t)i * nin], &x[(size_t)perm[i] * nin], nin * 4);
      std::memcpy(&ts[(size_t)i * nout], &t[(size_t)perm[i] * nout], nout * 4);
    }
    TTG_CUDA_TRY(cudaMemcpyAsync(dx.p, xs.data(), xs.size() * 4, cudaMemcpyHostToDevice, m->stream));
    TTG_CUDA_TRY(cudaMemcpyAsync(dt.p, ts.data(), ts.size() * 4, cudaMemcpyHostToDevice, m->stream));
    double ep_loss = 0.0;
    for (int b0 = 0; b0 + B <= n; b0 += B) {
      TTG_CUDA_TRY(cudaMemcpyAsync(H, dx.as<float>() + (size_t)b0 * nin, (size_t)B * nin * 4,
                                   cudaMemcpyDeviceToDevice, m->stream));
      TTG_CUDA_TRY(cudaMemcpyAsync(m->tbuf.p, dt.as<float>() + (size_t)b0 * nout,
                                   (size_t)B * nout * 4, cudaMemcpyDeviceToDevice, m->stream));
      ttg::forward(m, B);
      ep_loss += ttg::backward(m, B) * B;
      m->step++;
      const float c1 = 1.f - powf(0.9f, (float)m->step), c2 = 1.f - powf(0.999f, (float)m->step);
      ttg::k_adam<<<ttg::grid1(m->n_params), 256, 0, m->stream>>>(
          m->params.as<float>(), m->grads.as<float>(), m->m1.as<float>(), m->m2.as<float>(),
          m->n_params, lr, 0.9f, 0.999f, 1e-8f, c1, c2, weight_decay,
          mask.as<unsigned char>()); TTG_COUNT();
      TTG_CUDA_TRY(cudaGetLastError());
    }
    if (loss_per_epoch) loss_per_epoch[ep] = (float)(ep_loss / ((n / B) * B));
  }
  TTG_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return TTG_OK;
}

ttg_status ttg_atom_descriptors(int32_t natoms, const double* pos, int32_t n_features, double mu0,
                                double dmu, double eta, double rc, float* out) {
  if (natoms <= 0 || !pos || n_features <= 0 || !out || rc <= 0.0) return TTG_BAD_ARG;
  cudaStream_t st;
  TTG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamDefault));
  ttg_status s = TTG_OK;
  {
    ttg::DevBuf dp, dout;
    if ((s = dp.alloc((size_t)natoms * 3 * 8)) == TTG_OK &&
        (s = dout.alloc((size_t)natoms * n_features * 4)) == TTG_OK) {
      cudaMemcpyAsync(dp.p, pos, (size_t)natoms * 3 * 8, cudaMemcpyHostToDevice, st);
      ttg::k_descriptors<<<natoms, 64, 0, st>>>(dp.as<double>(), natoms, n_features, mu0, dmu,
                                                eta, rc, dout.as<float>()); TTG_COUNT();
      if (cudaGetLastError() != cudaSuccess) s = TTG_CUDA_ERR;
      else cudaMemcpyAsync(out, dout.p, (size_t)natoms * n_features * 4, cudaMemcpyDeviceToHost,
                           st);
    }
    cudaStreamSynchronize(st);
  }
  cudaStreamDestroy(st);
  return s;
}

}  // extern "C"
