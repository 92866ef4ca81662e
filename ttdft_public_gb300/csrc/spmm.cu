// Fused sparse-Hamiltonian SpMM + Chebyshev three-term update.
//
// One launch per filter degree computes, for every row i of the block,
//   Ynew[i,:] = alpha * ( sum_j H_loc[i,j] Y[j,:] + sum_a C[a,i] W[a,:] )
//             + beta * Y[i,:] + delta * X[i,:]
// which is the body of ChebyShevFilter::computeFilteredSubspace
// (eigensolver/ChebyShevFilter.cc:97-124 for the first degree, :129-170 for
// the others) with the H_loc product of AX::perform_ax
// (eigensolver/MultCuda.cu:719-820) and the nonlocal C_nloc_trans*(C_nloc*Y)
// product fused in.  W = diag(D) C Y is produced by a small reduction launch
// just before and stored as extra rows of the source block.
//
// Format: row groups of G consecutive rows share one merged, sorted column
// list (see RowGroups).  Rows of the Tucker basis are x-fastest, so G
// consecutive rows are neighbours along x and their column sets overlap
// almost completely; one load of Y[j,:] then feeds G rows (G FMAs per loaded
// element instead of 1 for CSR), which is what keeps the kernel off the
// L1/L2 gather limit.  Column indices and values of a group are contiguous
// in HBM, staged through shared memory in chunks with cp.async double
// buffering and read from there as warp-wide broadcasts.

#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ttg_internal.cuh"

namespace ttg {

ttg_status DevBuf::alloc(size_t n) {
  release();
  if (n == 0) return TTG_OK;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    return TTG_OOM;
  }
  bytes = n;
  return TTG_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

namespace {

// ---------------------------------------------------------------- loads ----

template <typename T, int VEC> struct Vec;
template <> struct Vec<double, 1> {
  static __device__ __forceinline__ void load(const double* p, double* v) { v[0] = __ldg(p); }
  static __device__ __forceinline__ void store(double* p, const double* v) { p[0] = v[0]; }
};
template <> struct Vec<double, 2> {
  static __device__ __forceinline__ void load(const double* p, double* v) {
    double2 t = __ldg(reinterpret_cast<const double2*>(p));
    v[0] = t.x; v[1] = t.y;
  }
  static __device__ __forceinline__ void store(double* p, const double* v) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  }
};
template <> struct Vec<float, 1> {
  static __device__ __forceinline__ void load(const float* p, float* v) { v[0] = __ldg(p); }
  static __device__ __forceinline__ void store(float* p, const float* v) { p[0] = v[0]; }
};
template <> struct Vec<float, 2> {
  static __device__ __forceinline__ void load(const float* p, float* v) {
    float2 t = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = t.x; v[1] = t.y;
  }
  static __device__ __forceinline__ void store(float* p, const float* v) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  }
};
template <> struct Vec<float, 4> {
  static __device__ __forceinline__ void load(const float* p, float* v) {
    float4 t = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static __device__ __forceinline__ void store(float* p, const float* v) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <> struct Vec<__nv_bfloat16, 2> {
  static __device__ __forceinline__ void load(const __nv_bfloat16* p, float* v) {
    unsigned u = __ldg(reinterpret_cast<const unsigned*>(p));
    __nv_bfloat162 t = *reinterpret_cast<__nv_bfloat162*>(&u);
    float2 f = __bfloat1622float2(t);
    v[0] = f.x; v[1] = f.y;
  }
  static __device__ __forceinline__ void store(__nv_bfloat16* p, const float* v) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v[0], v[1]);
  }
};
template <> struct Vec<__nv_bfloat16, 4> {
  static __device__ __forceinline__ void load(const __nv_bfloat16* p, float* v) {
    uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
    __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&u.x);
    __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&u.y);
    float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
    v[0] = fa.x; v[1] = fa.y; v[2] = fb.x; v[3] = fb.y;
  }
  static __device__ __forceinline__ void store(__nv_bfloat16* p, const float* v) {
    uint2 u;
    __nv_bfloat162 a = __floats2bfloat162_rn(v[0], v[1]);
    __nv_bfloat162 b = __floats2bfloat162_rn(v[2], v[3]);
    u.x = *reinterpret_cast<unsigned*>(&a);
    u.y = *reinterpret_cast<unsigned*>(&b);
    *reinterpret_cast<uint2*>(p) = u;
  }
};

template <typename T> __device__ __forceinline__ float to_acc(T v);
template <> __device__ __forceinline__ float to_acc<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_acc<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

// ------------------------------------------------------ cp.async helpers ----

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// ------------------------------------------------------- fused kernel ----
//
// CTA = one row group x all k columns.  Thread t owns columns
// [t*VEC, t*VEC+VEC).  Chunks of CH slots (column ids + G values each) are
// staged into shared memory with cp.async, two chunks in flight.
// Slot offsets of every group are multiples of 4, so each chunk's column ids
// (CH*4 bytes) and values (CH*G*sizeof(TV) bytes) are 16-byte aligned.

template <typename TV, typename TS, typename TA, int G, int VEC, int CH>
__global__ void __launch_bounds__(512) k_cheb_step(
    const int64_t* __restrict__ gptr, const int* __restrict__ gcol,
    const TV* __restrict__ gval, const TS* __restrict__ src, const TS* xold, TS* dst,
    int64_t n, int k, int64_t ld, TA alpha, TA beta, TA delta) {
  __shared__ __align__(16) int s_col[2][CH];
  __shared__ __align__(16) TV s_val[2][CH * G];
  const int64_t g = blockIdx.x;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int c0 = tid * VEC;
  const bool active = c0 < k;
  const int64_t s0 = gptr[g], s1 = gptr[g + 1];
  const int64_t nslots = s1 - s0;
  const int nchunks = (int)((nslots + CH - 1) / CH);

  auto stage = [&](int c, int buf) {
    const int64_t base = s0 + (int64_t)c * CH;
    const int cnt = (int)(s1 - base < CH ? s1 - base : CH);   // multiple of 4
    const int ncol16 = cnt / 4;                          // 16-byte pieces of column ids
    const int nval16 = cnt * G * (int)sizeof(TV) / 16;   // 16-byte pieces of values
    const char* gc = reinterpret_cast<const char*>(gcol + base);
    const char* gv = reinterpret_cast<const char*>(gval + base * G);
    char* sc = reinterpret_cast<char*>(s_col[buf]);
    char* sv = reinterpret_cast<char*>(s_val[buf]);
    for (int i = tid; i < ncol16 + nval16; i += nthr) {
      if (i < ncol16) cp_async16(sc + 16 * i, gc + 16 * i);
      else cp_async16(sv + 16 * (i - ncol16), gv + 16 * (i - ncol16));
    }
  };

  TA acc[G][VEC];
#pragma unroll
  for (int r = 0; r < G; ++r)
#pragma unroll
    for (int v = 0; v < VEC; ++v) acc[r][v] = TA(0);

  if (nchunks > 0) stage(0, 0);
  cp_async_commit();
  for (int c = 0; c < nchunks; ++c) {
    const int buf = c & 1;
    if (c + 1 < nchunks) stage(c + 1, buf ^ 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const int cnt = (int)(s1 - (s0 + (int64_t)c * CH) < CH ? s1 - (s0 + (int64_t)c * CH) : CH);
    if (active) {
      const TS* srcc = src + c0;
#pragma unroll 4
      for (int j = 0; j < cnt; ++j) {
        const int col = s_col[buf][j];
        TA xv[VEC];
        if constexpr (sizeof(TS) == sizeof(TA)) {
          Vec<TS, VEC>::load(srcc + (int64_t)col * ld, xv);
        } else {
          Vec<TS, VEC>::load(srcc + (int64_t)col * ld, xv);
        }
        const TV* hv = &s_val[buf][j * G];
#pragma unroll
        for (int r = 0; r < G; ++r) {
          TA h;
          if constexpr (sizeof(TV) == sizeof(TA)) h = hv[r];
          else h = to_acc<TV>(hv[r]);
#pragma unroll
          for (int v = 0; v < VEC; ++v) acc[r][v] = fma(h, xv[v], acc[r][v]);
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
#pragma unroll
  for (int r = 0; r < G; ++r) {
    const int64_t row = g * G + r;
    if (row >= n) break;
    TA y[VEC], o[VEC];
    Vec<TS, VEC>::load(src + row * ld + c0, y);
#pragma unroll
    for (int v = 0; v < VEC; ++v) o[v] = alpha * acc[r][v] + beta * y[v];
    if (delta != TA(0)) {
      TA x[VEC];
      Vec<TS, VEC>::load(xold + row * ld + c0, x);
#pragma unroll
      for (int v = 0; v < VEC; ++v) o[v] = fma(delta, x[v], o[v]);
    }
    Vec<TS, VEC>::store(dst + row * ld + c0, o);
  }
}

// Y = H X with FP64 values carried as unevaluated pairs of FP32 (hi + lo,
// ~44 significant bits), on the FP32 pipes.  Each product uses the exact
// FMA residual (a_hi*b_hi = p + fma(a_hi, b_hi, -p)) plus the two cross terms,
// and is accumulated with Knuth's error-free two-sum into (hi, lo).  GB300
// runs FP32 at many times its FP64 rate, so this carries the Rayleigh-Ritz
// product H X at FP64-level accuracy several times faster than FP64 FMAs.
// Source rows are float2 (hi, lo) pairs; H slots are float2 pairs too.
template <int G>
__global__ void __launch_bounds__(512) k_apply_df64(
    const int64_t* __restrict__ gptr, const int* __restrict__ gcol,
    const float2* __restrict__ gval, const float2* __restrict__ src, double* __restrict__ dst,
    int64_t n, int k, int64_t ld) {
  constexpr int CH = 32;
  __shared__ __align__(16) int s_col[2][CH];
  __shared__ __align__(16) float2 s_val[2][CH * G];
  const int64_t g = blockIdx.x;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int c0 = blockIdx.y * blockDim.x + tid;       // state (column) of this thread
  const bool active = c0 < k;
  const int64_t s0 = gptr[g], s1 = gptr[g + 1];
  const int nchunks = (int)((s1 - s0 + CH - 1) / CH);
  auto stage = [&](int c, int buf) {
    const int64_t base = s0 + (int64_t)c * CH;
    const int cnt = (int)(s1 - base < CH ? s1 - base : CH);   // multiple of 4
    const int ncol16 = cnt / 4;
    const int nval16 = cnt * G * 8 / 16;
    const char* gc = reinterpret_cast<const char*>(gcol + base);
    const char* gv = reinterpret_cast<const char*>(gval + base * G);
    char* sc = reinterpret_cast<char*>(s_col[buf]);
    char* sv = reinterpret_cast<char*>(s_val[buf]);
    for (int i = tid; i < ncol16 + nval16; i += nthr) {
      if (i < ncol16) cp_async16(sc + 16 * i, gc + 16 * i);
      else cp_async16(sv + 16 * (i - ncol16), gv + 16 * (i - ncol16));
    }
  };
  float hi[G], lo[G];
#pragma unroll
  for (int r = 0; r < G; ++r) hi[r] = lo[r] = 0.f;
  if (nchunks > 0) stage(0, 0);
  cp_async_commit();
  for (int c = 0; c < nchunks; ++c) {
    const int buf = c & 1;
    if (c + 1 < nchunks) stage(c + 1, buf ^ 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const int cnt = (int)(s1 - (s0 + (int64_t)c * CH) < CH ? s1 - (s0 + (int64_t)c * CH) : CH);
    if (active) {
#pragma unroll 2
      for (int j = 0; j < cnt; ++j) {
        const float2 x = __ldg(src + (int64_t)s_col[buf][j] * ld + c0);
        const float2* hv = &s_val[buf][j * G];
#pragma unroll
        for (int r = 0; r < G; ++r) {
          const float2 h = hv[r];
          // about half of a group's slots are zero for a given row; every
          // thread of the CTA sees the same value, so the skip is uniform
          if (h.x == 0.f) continue;
          const float p = h.x * x.x;
          float e = fmaf(h.x, x.x, -p);
          e = fmaf(h.x, x.y, e);
          e = fmaf(h.y, x.x, e);
          const float s = hi[r] + p;
          const float bb = s - hi[r];
          const float err = (hi[r] - (s - bb)) + (p - bb);
          hi[r] = s;
          lo[r] += err + e;
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
#pragma unroll
  for (int r = 0; r < G; ++r) {
    const int64_t row = g * G + r;
    if (row < n) dst[row * ld + c0] = (double)hi[r] + (double)lo[r];
  }
}

__global__ void k_split_df64(const double* __restrict__ src, float2* __restrict__ dst,
                             int64_t rows, int k, int64_t ld) {
  const int64_t total = rows * (int64_t)k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / k;
    const int c = (int)(i - r * k);
    const double v = src[r * ld + c];
    const float h = __double2float_rn(v);
    dst[r * ld + c] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

__global__ void k_split_vals(const double* __restrict__ src, float2* __restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = src[i];
    const float h = __double2float_rn(v);
    dst[i] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

// k == 1 (Lanczos SpMV): one warp per row group, lanes split the slots.
template <int G>
__global__ void k_spmv_rg(const int64_t* __restrict__ gptr, const int* __restrict__ gcol,
                          const double* __restrict__ gval, const double* __restrict__ src,
                          double* dst, int64_t n, int64_t n_groups, int64_t ld, double alpha,
                          double beta) {
  const int lane = threadIdx.x & 31;
  const int64_t g = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (g >= n_groups) return;
  double acc[G];
#pragma unroll
  for (int r = 0; r < G; ++r) acc[r] = 0.0;
  for (int64_t s = gptr[g] + lane; s < gptr[g + 1]; s += 32) {
    const double x = __ldg(src + (int64_t)gcol[s] * ld);
#pragma unroll
    for (int r = 0; r < G; ++r) acc[r] = fma(gval[s * G + r], x, acc[r]);
  }
#pragma unroll
  for (int r = 0; r < G; ++r)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
  if (lane < G) {
    double a = acc[0];
#pragma unroll
    for (int r = 1; r < G; ++r)
      if (lane == r) a = acc[r];
    const int64_t row = g * G + lane;
    if (row < n) dst[row * ld] = alpha * a + beta * src[row * ld];
  }
}

// W[a,:] = sum_J Cd[a,J] Y[J,:] (Cd = diag(D) C), written to row n + a of the
// source block.  Two launches so that all SMs take part: (1) grid (nproj,
// splits): each CTA sums kProjChunk entries of one projector row into a
// partial row; (2) the partial rows are summed in a fixed order (bitwise
// reproducible) and stored.
constexpr int kProjChunk = 128;

template <typename TS, typename TA>
__global__ void k_proj_partial(const int64_t* __restrict__ cptr, const int* __restrict__ ccol,
                               const double* __restrict__ cval, const TS* __restrict__ src, int k,
                               int64_t ld, TA* __restrict__ part, int nsplit) {
  const int a = blockIdx.x, sp = blockIdx.y;
  const int64_t e0 = cptr[a] + (int64_t)sp * kProjChunk;
  const int64_t e1 = min(cptr[a + 1], e0 + kProjChunk);
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    TA acc = TA(0);
    for (int64_t e = e0; e < e1; ++e) {
      TA x;
      if constexpr (sizeof(TS) == sizeof(TA)) x = src[(int64_t)ccol[e] * ld + c];
      else x = to_acc<TS>(src[(int64_t)ccol[e] * ld + c]);
      acc = fma((TA)cval[e], x, acc);
    }
    part[((int64_t)a * nsplit + sp) * k + c] = acc;
  }
}

template <typename TS, typename TA>
__global__ void k_proj_reduce(const TA* __restrict__ part, int nsplit, TS* src, int64_t n, int k,
                              int64_t ld) {
  const int a = blockIdx.x;
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    TA s = TA(0);
    for (int sp = 0; sp < nsplit; ++sp) s += part[((int64_t)a * nsplit + sp) * k + c];
    if constexpr (sizeof(TS) == sizeof(TA)) src[(n + a) * ld + c] = s;
    else src[(n + a) * ld + c] = __float2bfloat16_rn((float)s);
  }
}

template <typename TI, typename TO>
__device__ __forceinline__ TO cvt(TI v) { return (TO)v; }
template <> __device__ __forceinline__ __nv_bfloat16 cvt<double, __nv_bfloat16>(double v) {
  return __double2bfloat16(v);
}
template <> __device__ __forceinline__ __nv_bfloat16 cvt<float, __nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
template <> __device__ __forceinline__ float cvt<__nv_bfloat16, float>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}
template <> __device__ __forceinline__ double cvt<__nv_bfloat16, double>(__nv_bfloat16 v) {
  return (double)__bfloat162float(v);
}

template <typename TI, typename TO>
__global__ void k_convert_rows(const TI* __restrict__ src, TO* __restrict__ dst, int64_t rows,
                               int k, int64_t ld) {
  const int64_t total = rows * (int64_t)k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / k;
    const int c = (int)(i - r * k);
    dst[r * ld + c] = cvt<TI, TO>(src[r * ld + c]);
  }
}

template <typename TO>
__global__ void k_convert_vals(const double* __restrict__ src, TO* __restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = cvt<double, TO>(src[i]);
}

__global__ void k_scale_rows_f64(double* v, const double* d, const int64_t* ptr, int nrows) {
  const int a = blockIdx.x;
  for (int64_t e = ptr[a] + threadIdx.x; e < ptr[a + 1]; e += blockDim.x) v[e] *= d[a];
}

int grid_for(int64_t work, int threads) {
  int64_t b = (work + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

// ------------------------------------------------------------- host side --

static ttg_status validate_csr(int64_t rows, int64_t cols, const int64_t* p, const int32_t* c,
                               const double* v) {
  if (rows < 0 || !p) return TTG_BAD_ARG;
  if (p[0] != 0) return TTG_BAD_CSR;
  for (int64_t i = 0; i < rows; ++i)
    if (p[i + 1] < p[i]) return TTG_BAD_CSR;
  const int64_t nnz = p[rows];
  if (nnz > 0 && (!c || !v)) return TTG_BAD_ARG;
  int bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
  for (int64_t i = 0; i < rows; ++i)
    for (int64_t e = p[i]; e < p[i + 1]; ++e) {
      if (c[e] < 0 || c[e] >= cols) bad |= 1;
      if (e > p[i] && c[e] <= c[e - 1]) bad |= 1;   // sorted, unique
      if (!std::isfinite(v[e])) bad |= 2;
    }
  if (bad & 2) return TTG_NONFINITE;
  if (bad) return TTG_BAD_CSR;
  return TTG_OK;
}

ttg_status build_row_groups(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                            const double* hv, int32_t nproj, const int64_t* cp,
                            const int32_t* cc, const double* cv, const double* d) {
  constexpr int G = kGroupRows;
  TTG_TRY(validate_csr(n, n, hp, hc, hv));
  if (nproj > 0) {
    TTG_TRY(validate_csr(nproj, n, cp, cc, cv));
    if (!d) return TTG_BAD_ARG;
    for (int a = 0; a < nproj; ++a)
      if (!std::isfinite(d[a])) return TTG_NONFINITE;
  }
  // C^T rows: for each basis row i, the (a, C[a,i]) pairs, a ascending.
  std::vector<int64_t> tp(n + 1, 0);
  std::vector<int32_t> tc;
  std::vector<double> tv;
  if (nproj > 0) {
    for (int a = 0; a < nproj; ++a)
      for (int64_t e = cp[a]; e < cp[a + 1]; ++e) tp[cc[e] + 1]++;
    for (int64_t i = 0; i < n; ++i) tp[i + 1] += tp[i];
    tc.resize(tp[n]);
    tv.resize(tp[n]);
    std::vector<int64_t> fillp(tp.begin(), tp.end() - 1);
    for (int a = 0; a < nproj; ++a)
      for (int64_t e = cp[a]; e < cp[a + 1]; ++e) {
        const int64_t i = cc[e];
        tc[fillp[i]] = (int32_t)(n + a);
        tv[fillp[i]] = cv[e];
        fillp[i]++;
      }
  }
  const int64_t ng = (n + G - 1) / G;
  std::vector<int64_t> gptr(ng + 1, 0);
  // merged, sorted column list of one group (H part then C^T part)
  auto merge = [&](int64_t g, std::vector<int32_t>& out) {
    out.clear();
    const int64_t r0 = g * G, r1 = std::min<int64_t>(n, r0 + G);
    int64_t pos[2][G];
    for (int pass = 0; pass < 2; ++pass) {
      const int64_t* P = pass == 0 ? hp : tp.data();
      const int32_t* Cc = pass == 0 ? hc : tc.data();
      for (int64_t r = r0; r < r1; ++r) pos[pass][r - r0] = P[r];
      while (true) {
        int32_t mn = INT32_MAX;
        for (int64_t r = r0; r < r1; ++r)
          if (pos[pass][r - r0] < P[r + 1]) mn = std::min(mn, Cc[pos[pass][r - r0]]);
        if (mn == INT32_MAX) break;
        out.push_back(mn);
        for (int64_t r = r0; r < r1; ++r)
          if (pos[pass][r - r0] < P[r + 1] && Cc[pos[pass][r - r0]] == mn) pos[pass][r - r0]++;
      }
    }
  };
#pragma omp parallel
  {
    std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 16)
    for (int64_t g = 0; g < ng; ++g) {
      merge(g, cols);
      gptr[g + 1] = ((int64_t)cols.size() + 3) / 4 * 4;
    }
  }
  for (int64_t g = 0; g < ng; ++g) gptr[g + 1] += gptr[g];
  const int64_t slots = gptr[ng];
  std::vector<int32_t> gcol(slots);
  std::vector<double> gval(slots * G, 0.0);
  // position of every H_loc entry in the value array (for value updates)
  std::vector<int32_t> rgpos(op->keep_pattern ? hp[n] : 0);
#pragma omp parallel
  {
    std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 16)
    for (int64_t g = 0; g < ng; ++g) {
      merge(g, cols);
      const int64_t base = gptr[g];
      const int64_t cnt = (int64_t)cols.size();
      for (int64_t s = 0; s < gptr[g + 1] - base; ++s)
        gcol[base + s] = cols.empty() ? 0 : cols[std::min<int64_t>(s, cnt - 1)];
      const int64_t r0 = g * G, r1 = std::min<int64_t>(n, r0 + G);
      for (int64_t r = r0; r < r1; ++r) {
        // walk the row's entries along the merged list (both sorted)
        int64_t s = 0;
        for (int64_t e = hp[r]; e < hp[r + 1]; ++e) {
          while (cols[s] != hc[e]) ++s;
          gval[(base + s) * G + (r - r0)] = hv[e];
          if (!rgpos.empty()) rgpos[e] = (int32_t)s;   // slot within the group
        }
        if (nproj > 0)
          for (int64_t e = tp[r]; e < tp[r + 1]; ++e) {
            while (cols[s] != tc[e]) ++s;
            gval[(base + s) * G + (r - r0)] = tv[e];
          }
      }
    }
  }
  RowGroups& rg = op->rg;
  rg.n_groups = ng;
  rg.slots = slots;
  TTG_TRY(rg.gptr.alloc((ng + 1) * sizeof(int64_t)));
  TTG_TRY(rg.gcol.alloc(std::max<int64_t>(slots, 4) * sizeof(int32_t)));
  TTG_TRY(rg.v64.alloc(std::max<int64_t>(slots, 4) * G * sizeof(double)));

  TTG_CUDA_TRY(cudaMemcpyAsync(rg.gptr.p, gptr.data(), (ng + 1) * sizeof(int64_t),
                               cudaMemcpyHostToDevice, op->stream));
  if (slots > 0) {
    TTG_CUDA_TRY(cudaMemcpyAsync(rg.gcol.p, gcol.data(), slots * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, op->stream));
    TTG_CUDA_TRY(cudaMemcpyAsync(rg.v64.p, gval.data(), slots * G * sizeof(double),
                                 cudaMemcpyHostToDevice, op->stream));

  }
  // C with D folded in (C_nloc = diag(D) C), plus an FP32 copy
  Csr& C = op->C;
  C.rows = nproj;
  C.cols = n;
  C.nnz = nproj > 0 ? cp[nproj] : 0;
  C.max_row_nnz = 0;
  for (int a = 0; a < nproj; ++a) C.max_row_nnz = std::max<int64_t>(C.max_row_nnz, cp[a + 1] - cp[a]);
  if (nproj > 0) {
    TTG_TRY(C.ptr.alloc((nproj + 1) * sizeof(int64_t)));
    TTG_TRY(C.col.alloc(std::max<int64_t>(C.nnz, 1) * sizeof(int32_t)));
    TTG_TRY(C.val.alloc(std::max<int64_t>(C.nnz, 1) * sizeof(double)));
    std::vector<double> dv(C.nnz);
    for (int a = 0; a < nproj; ++a)
      for (int64_t e = cp[a]; e < cp[a + 1]; ++e) dv[e] = d[a] * cv[e];
    TTG_CUDA_TRY(cudaMemcpyAsync(C.ptr.p, cp, (nproj + 1) * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, op->stream));
    if (C.nnz > 0) {
      TTG_CUDA_TRY(cudaMemcpyAsync(C.col.p, cc, C.nnz * sizeof(int32_t), cudaMemcpyHostToDevice,
                                   op->stream));
      TTG_CUDA_TRY(cudaMemcpyAsync(C.val.p, dv.data(), C.nnz * sizeof(double),
                                   cudaMemcpyHostToDevice, op->stream));
    }
  }
  op->nnz_h = hp[n];
  op->nnz_c = C.nnz;
  if (op->keep_pattern && hp[n] > 0) {
    Pattern& P = op->pattern;
    // half-bandwidth of the pattern in each Tucker direction
    const int rx = P.r[0], ry = P.r[1];
    int bx = 0, by = 0, bz = 0;
#pragma omp parallel for reduction(max : bx, by, bz) schedule(static)
    for (int64_t I = 0; I < n; ++I) {
      const int xI = (int)(I % rx), yI = (int)((I / rx) % ry), zI = (int)(I / ((int64_t)rx * ry));
      for (int64_t e = hp[I]; e < hp[I + 1]; ++e) {
        const int J = hc[e];
        bx = std::max(bx, std::abs(J % rx - xI));
        by = std::max(by, std::abs((J / rx) % ry - yI));
        bz = std::max(bz, std::abs(J / (rx * ry) - zI));
      }
    }
    P.bw[0] = bx;
    P.bw[1] = by;
    P.bw[2] = bz;
    TTG_TRY(P.row_ptr.alloc((n + 1) * sizeof(int64_t)));
    TTG_TRY(P.col.alloc(hp[n] * sizeof(int32_t)));
    TTG_TRY(P.rg_pos.alloc(hp[n] * sizeof(int32_t)));
    TTG_CUDA_TRY(cudaMemcpyAsync(P.row_ptr.p, hp, (n + 1) * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, op->stream));
    TTG_CUDA_TRY(cudaMemcpyAsync(P.col.p, hc, hp[n] * sizeof(int32_t), cudaMemcpyHostToDevice,
                                 op->stream));
    TTG_CUDA_TRY(cudaMemcpyAsync(P.rg_pos.p, rgpos.data(), hp[n] * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, op->stream));
    op->device_bytes += P.row_ptr.bytes + P.col.bytes + P.rg_pos.bytes;
  }
  // host vectors above are freed on return: wait for the copies
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  op->device_bytes += rg.gptr.bytes + rg.gcol.bytes + rg.v64.bytes + C.ptr.bytes + C.col.bytes +
                      C.val.bytes;
  return TTG_OK;
}

// FP32 / BF16 / (hi, lo) copies of the row-group values, made from the FP64
// values on first use (the tensor-core format serves the FP32 and BF16
// degrees, so these are needed only for block widths it does not take).
static ttg_status rg_values(ttg_op* op, int prec, void** out) {
  RowGroups& rg = op->rg;
  const int64_t cnt = std::max<int64_t>(rg.slots, 4) * kGroupRows;
  const int grid = grid_for(cnt, 256);
  if (prec == TTG_PREC_FP32 && !rg.v32.p) {
    TTG_TRY(rg.v32.alloc(cnt * sizeof(float)));
    k_convert_vals<float><<<grid, 256, 0, op->stream>>>(rg.v64.as<double>(), rg.v32.as<float>(), cnt); TTG_COUNT();
    TTG_LAUNCHED(op);
    op->device_bytes += rg.v32.bytes;
  } else if (prec == TTG_PREC_BF16 && !rg.v16.p) {
    TTG_TRY(rg.v16.alloc(cnt * sizeof(__nv_bfloat16)));
    k_convert_vals<__nv_bfloat16><<<grid, 256, 0, op->stream>>>(rg.v64.as<double>(),
                                                               rg.v16.as<__nv_bfloat16>(), cnt); TTG_COUNT();
    TTG_LAUNCHED(op);
    op->device_bytes += rg.v16.bytes;
  } else if (prec == TTG_PREC_DF64 && !rg.vdf.p) {
    TTG_TRY(rg.vdf.alloc(cnt * sizeof(float2)));
    k_split_vals<<<grid, 256, 0, op->stream>>>(rg.v64.as<double>(), rg.vdf.as<float2>(), cnt); TTG_COUNT();
    TTG_LAUNCHED(op);
    op->device_bytes += rg.vdf.bytes;
  }
  *out = prec == TTG_PREC_FP32 ? rg.v32.p : prec == TTG_PREC_BF16 ? rg.v16.p
         : prec == TTG_PREC_DF64 ? rg.vdf.p : rg.v64.p;
  return TTG_OK;
}

template <typename TV, typename TS, typename TA, int VEC>
static ttg_status launch_step_t(ttg_op* op, const TV* vals, const void* src, const void* xold,
                                void* dst, int k, double alpha, double beta, double delta) {
  constexpr int G = kGroupRows;
  constexpr int CH = sizeof(TV) == 8 ? 32 : 64;
  int threads = (k + VEC - 1) / VEC;
  threads = (threads + 31) / 32 * 32;
  if (threads > 512) return TTG_BAD_ARG;
  if (op->rg.n_groups == 0) return TTG_OK;
  TTG_TRY(kt_begin(op, TTG_KT_ROWGROUP));
  k_cheb_step<TV, TS, TA, G, VEC, CH><<<(unsigned)op->rg.n_groups, threads, 0, op->stream>>>(
      op->rg.gptr.as<int64_t>(), op->rg.gcol.as<int>(), vals,
      reinterpret_cast<const TS*>(src), reinterpret_cast<const TS*>(xold),
      reinterpret_cast<TS*>(dst), op->n, k, op->ld, (TA)alpha, (TA)beta, (TA)delta); TTG_COUNT();
  TTG_LAUNCHED(op);
  TTG_TRY(kt_end(op));
  return TTG_OK;
}

ttg_status launch_cheb_step(ttg_op* op, int prec, const void* src, const void* xold, void* dst,
                            int k, double alpha, double beta, double delta) {
  if (k <= 0 || k > op->max_k) return TTG_BAD_ARG;
  if (umma_supported(op, prec, k))
    return launch_cheb_umma(op, prec, src, xold, dst, k, alpha, beta, delta);
  // blocks wider than one MMA (N <= 256): the tcgen05 degree over column
  // blocks of at most 256 states, each re-reading H (the reference's
  // num_X_blocks, ChebyShevFilter.cc:97-170, splits its columns the same way)
  if (k > 256 && k % 16 == 0 && umma_supported(op, prec, 256)) {
    const int nblk = (k + 255) / 256;
    const int kb = ((k + nblk - 1) / nblk + 15) / 16 * 16;
    const size_t elem = prec == TTG_PREC_FP32 ? 4 : 2;
    for (int c0 = 0; c0 < k; c0 += kb) {
      const int kk = std::min(kb, k - c0);
      TTG_TRY(launch_cheb_umma(op, prec, static_cast<const char*>(src) + c0 * elem,
                               xold ? static_cast<const char*>(xold) + c0 * elem : nullptr,
                               static_cast<char*>(dst) + c0 * elem, kk, alpha, beta, delta));
    }
    return TTG_OK;
  }
  if (tc_supported(op, prec, k))
    return launch_cheb_tc(op, prec, src, xold, dst, k, alpha, beta, delta);
  if (prec == TTG_PREC_FP64) {
    if (k == 1) {
      const int wpb = 8;
      const int blocks = (int)((op->rg.n_groups + wpb - 1) / wpb);
      if (delta != 0.0) return TTG_BAD_ARG;
      k_spmv_rg<kGroupRows><<<blocks, 32 * wpb, 0, op->stream>>>(
          op->rg.gptr.as<int64_t>(), op->rg.gcol.as<int>(), op->rg.v64.as<double>(),
          reinterpret_cast<const double*>(src), reinterpret_cast<double*>(dst), op->n,
          op->rg.n_groups, op->ld, alpha, beta); TTG_COUNT();
      TTG_LAUNCHED(op);
      return TTG_OK;
    }
    if (k % 2 == 0 && k <= 1024)
      return launch_step_t<double, double, double, 2>(op, op->rg.v64.as<double>(), src, xold,
                                                      dst, k, alpha, beta, delta);
    return launch_step_t<double, double, double, 1>(op, op->rg.v64.as<double>(), src, xold, dst,
                                                    k, alpha, beta, delta);
  }
  if (prec == TTG_PREC_FP32 || prec == TTG_PREC_BF16) {
    void* vp = nullptr;
    TTG_TRY(rg_values(op, prec, &vp));
  }
  if (prec == TTG_PREC_FP32) {
    if (k % 4 == 0 && k > 256)
      return launch_step_t<float, float, float, 4>(op, op->rg.v32.as<float>(), src, xold, dst, k,
                                                   alpha, beta, delta);
    if (k % 2 == 0)
      return launch_step_t<float, float, float, 2>(op, op->rg.v32.as<float>(), src, xold, dst, k,
                                                   alpha, beta, delta);
    return launch_step_t<float, float, float, 1>(op, op->rg.v32.as<float>(), src, xold, dst, k,
                                                 alpha, beta, delta);
  }
  if (prec == TTG_PREC_BF16) {
    if (k % 4 == 0)
      return launch_step_t<__nv_bfloat16, __nv_bfloat16, float, 4>(
          op, op->rg.v16.as<__nv_bfloat16>(), src, xold, dst, k, alpha, beta, delta);
    if (k % 2 == 0)
      return launch_step_t<__nv_bfloat16, __nv_bfloat16, float, 2>(
          op, op->rg.v16.as<__nv_bfloat16>(), src, xold, dst, k, alpha, beta, delta);
    return TTG_BAD_ARG;
  }
  return TTG_BAD_ARG;
}

ttg_status launch_apply_df64(ttg_op* op, const double* src, double* dst, int k) {
  if (k <= 0 || k > op->max_k) return TTG_BAD_ARG;
  const size_t need = (size_t)(op->n + op->nproj) * op->ld * sizeof(float2);
  if (op->wdf.bytes < need) {
    TTG_TRY(op->wdf.alloc(need));
    op->device_bytes += need;
  }
  void* vdf = nullptr;
  TTG_TRY(rg_values(op, TTG_PREC_DF64, &vdf));
  const int64_t rows = op->n + op->nproj;
  k_split_df64<<<grid_for(rows * k, 256), 256, 0, op->stream>>>(src, op->wdf.as<float2>(), rows,
                                                                k, op->ld); TTG_COUNT();
  TTG_LAUNCHED(op);
  if (op->rg.n_groups == 0) return TTG_OK;
  const int threads = std::min(512, (k + 31) / 32 * 32);
  dim3 grid((unsigned)op->rg.n_groups, (unsigned)((k + threads - 1) / threads));
  k_apply_df64<kGroupRows><<<grid, threads, 0, op->stream>>>(
      op->rg.gptr.as<int64_t>(), op->rg.gcol.as<int>(), op->rg.vdf.as<float2>(),
      op->wdf.as<float2>(), dst, op->n, k, op->ld); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

template <typename TS, typename TA>
static ttg_status proj_w_t(ttg_op* op, TS* src, int k) {
  const int nsplit = (int)((op->C.max_row_nnz + kProjChunk - 1) / kProjChunk);
  if (nsplit == 0) return TTG_OK;
  const size_t need = (size_t)op->nproj * nsplit * k * sizeof(TA);
  if (op->wpart.bytes < need) {
    TTG_TRY(op->wpart.alloc(need));
    op->device_bytes += need;
  }
  const int threads = std::min(256, (k + 31) / 32 * 32);
  k_proj_partial<TS, TA><<<dim3(op->nproj, nsplit), threads, 0, op->stream>>>(
      op->C.ptr.as<int64_t>(), op->C.col.as<int>(), op->C.val.as<double>(), src, k, op->ld,
      op->wpart.as<TA>(), nsplit); TTG_COUNT();
  TTG_LAUNCHED(op);
  k_proj_reduce<TS, TA><<<op->nproj, threads, 0, op->stream>>>(op->wpart.as<TA>(), nsplit, src,
                                                              op->n, k, op->ld); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status launch_proj_w(ttg_op* op, int prec, void* src, int k) {
  if (op->nproj == 0) return TTG_OK;
  if (prec == TTG_PREC_FP64) return proj_w_t<double, double>(op, reinterpret_cast<double*>(src), k);
  if (prec == TTG_PREC_FP32) return proj_w_t<float, float>(op, reinterpret_cast<float*>(src), k);
  return proj_w_t<__nv_bfloat16, float>(op, reinterpret_cast<__nv_bfloat16*>(src), k);
}

ttg_status launch_convert(ttg_op* op, int from, int to, const void* src, void* dst, int64_t rows,
                          int k) {
  const int grid = grid_for(rows * k, 256);
  if (from == TTG_PREC_FP64 && to == TTG_PREC_FP32)
    k_convert_rows<double, float><<<grid, 256, 0, op->stream>>>(
        (const double*)src, (float*)dst, rows, k, op->ld);
  else if (from == TTG_PREC_FP64 && to == TTG_PREC_BF16)
    k_convert_rows<double, __nv_bfloat16><<<grid, 256, 0, op->stream>>>(
        (const double*)src, (__nv_bfloat16*)dst, rows, k, op->ld);
  else if (from == TTG_PREC_FP32 && to == TTG_PREC_FP64)
    k_convert_rows<float, double><<<grid, 256, 0, op->stream>>>(
        (const float*)src, (double*)dst, rows, k, op->ld);
  else if (from == TTG_PREC_BF16 && to == TTG_PREC_FP32)
    k_convert_rows<__nv_bfloat16, float><<<grid, 256, 0, op->stream>>>(
        (const __nv_bfloat16*)src, (float*)dst, rows, k, op->ld);
  else if (from == TTG_PREC_BF16 && to == TTG_PREC_FP64)
    k_convert_rows<__nv_bfloat16, double><<<grid, 256, 0, op->stream>>>(
        (const __nv_bfloat16*)src, (double*)dst, rows, k, op->ld);
  else
    return TTG_BAD_ARG;
  TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

}  // namespace ttg
