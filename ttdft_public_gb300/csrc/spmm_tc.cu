// Tensor-core fused SpMM + Chebyshev update for the FP32 and BF16 degrees.
//
// Same recurrence as spmm.cu (ChebyShevFilter.cc:97-170), a different
// operator format:
//
// Row tiles.  The 64 rows of a tile are a 4 x 4 x 4 block of the Tucker
// index (x, y, z), I = x + rx*(y + ry*z).  The Hamiltonian couples a basis
// function only to neighbours in all three directions, so the rows of a 3-D
// block share most of their columns: each gathered row of the source block
// feeds 64 output rows (at fill ~0.3) instead of 8.  Generic CSR input without
// Tucker dimensions falls back to tiles of 64 consecutive rows.
//
// Per tile the sorted union of the rows' columns is stored in slots, padded to
// whole chunks of 16; each chunk holds the 16 x 64 block of H values already
// arranged in the register order of the MMA B operand (one 16-byte read per
// lane per 8-row n-tile for TF32, one 8-byte read for BF16).  Each chunk's H
// block and its 16 gathered source rows are staged together into shared
// memory with cp.async (3 stages in flight for FP32, 4 for BF16); the rows
// are the MMA A operand: the product is computed transposed,
// D[states x rows] = X^T[states x slots] H^T[slots x rows].
//
// FP32 degrees use three TF32 MMAs per tile (hi*hi + hi*lo + lo*hi, the
// split made in registers), which keeps FP32-level accuracy; BF16 degrees use
// one m16n8k16 BF16 MMA with the A operand loaded by ldmatrix.trans.
// Accumulation is FP32 in both.

#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include <type_traits>

#include "ttg_internal.cuh"

namespace ttg {
namespace {

constexpr int TR = 64;       // rows per tile
constexpr int CS = 16;       // slots per chunk

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ uint32_t tf32_of(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_of(x);
  lo = tf32_of(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t* r, const void* smem) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}

template <typename T> struct TcTraits;
template <> struct TcTraits<float> {
  static constexpr int PAD = 8;     // row pitch = 8 (mod 32) floats: conflict-free A loads
  static constexpr int VEC = 4;     // elements per 16-byte gather piece
  static constexpr int STAGES = 3;
  using HV = float4;                // per-lane H fragment of one chunk and n-tile
};
template <> struct TcTraits<__nv_bfloat16> {
  static constexpr int PAD = 8;     // row pitch = 8 (mod 16) elements: conflict-free ldmatrix
  static constexpr int VEC = 8;
  static constexpr int STAGES = 4;
  using HV = uint2;
};

// CTA: one tile (64 rows) x KS = 32*MT states; 4 warps = 2 (row halves) x
// 2 (state halves); each warp owns 4 n-tiles (32 rows) x MT m-tiles.
template <typename T, int MT>
__global__ void __launch_bounds__(128) k_cheb_tc(
    const int64_t* __restrict__ tptr, const int* __restrict__ tcol, const int* __restrict__ rowmap,
    const typename TcTraits<T>::HV* __restrict__ hval, const T* __restrict__ src, const T* xold,
    T* dst, int k, int64_t ld, float alpha, float beta, float delta) {
  using Tr = TcTraits<T>;
  using HV = typename Tr::HV;
  constexpr int STAGES = Tr::STAGES;
  constexpr int KS = 32 * MT;
  constexpr int SP = KS + Tr::PAD;
  constexpr int PIECES = CS * KS / Tr::VEC;
  constexpr int HPIECES = 8 * 32 * (int)sizeof(HV) / 16;   // H fragments of one chunk
  __shared__ __align__(16) T sX[STAGES][CS][SP];
  __shared__ __align__(16) HV sH[STAGES][8 * 32];

  const int tile = blockIdx.x;
  const int s_base = blockIdx.y * KS;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, tt = lane & 3;
  const int wn = warp & 1, wm = warp >> 1;
  const int64_t c_first = tptr[tile] / CS;
  const int nchunks = (int)((tptr[tile + 1] - tptr[tile]) / CS);

  auto gather = [&](int c, int stage) {
    const int* cols = tcol + (c_first + c) * CS;
    const char* hsrc = reinterpret_cast<const char*>(hval + (c_first + c) * 8 * 32);
    char* hdst = reinterpret_cast<char*>(&sH[stage][0]);
    for (int p = tid; p < HPIECES; p += 128) cp_async16(hdst + 16 * p, hsrc + 16 * p);
#pragma unroll
    for (int p = tid; p < PIECES; p += 128) {
      const int j = p / (KS / Tr::VEC);
      const int q = p - j * (KS / Tr::VEC);
      const int state = s_base + q * Tr::VEC;
      T* d = &sX[stage][j][q * Tr::VEC];
      if (state < k) {
        cp_async16(d, src + (int64_t)__ldg(cols + j) * ld + state);
      } else {
        *reinterpret_cast<uint4*>(d) = make_uint4(0, 0, 0, 0);
      }
    }
  };

  float acc[MT][4][4];
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  // prologue: STAGES-1 chunks in flight
#pragma unroll
  for (int s = 0; s < STAGES - 1; ++s) {
    if (s < nchunks) gather(s, s);
    cp_async_commit();
  }
  HV hv[4];
  for (int c = 0; c < nchunks; ++c) {
    const int stage = c % STAGES;
    if (c + STAGES - 1 < nchunks) gather(c + STAGES - 1, (c + STAGES - 1) % STAGES);
    cp_async_commit();
    cp_async_wait<STAGES - 1>();
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) hv[j] = sH[stage][(wn * 4 + j) * 32 + lane];
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        uint32_t bh[4][2], bl[4][2];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float b0 = ks == 0 ? hv[j].x : hv[j].z;
          const float b1 = ks == 0 ? hv[j].y : hv[j].w;
          split(b0, bh[j][0], bl[j][0]);
          split(b1, bh[j][1], bl[j][1]);
        }
#pragma unroll
        for (int i = 0; i < MT; ++i) {
          const int m0 = (wm * MT + i) * 16;
          uint32_t ah[4], al[4];
          split(sX[stage][ks * 8 + tt][m0 + g], ah[0], al[0]);
          split(sX[stage][ks * 8 + tt][m0 + g + 8], ah[1], al[1]);
          split(sX[stage][ks * 8 + tt + 4][m0 + g], ah[2], al[2]);
          split(sX[stage][ks * 8 + tt + 4][m0 + g + 8], ah[3], al[3]);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            mma_tf32(acc[i][j], al, bh[j][0], bh[j][1]);
            mma_tf32(acc[i][j], ah, bl[j][0], bl[j][1]);
            mma_tf32(acc[i][j], ah, bh[j][0], bh[j][1]);
          }
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < MT; ++i) {
        const int m0 = (wm * MT + i) * 16;
        const int quad = lane >> 3;
        const T* p = &sX[stage][(quad >> 1) * 8 + (lane & 7)][m0 + (quad & 1) * 8];
        uint32_t a[4];
        ldmatrix_x4_trans(a, p);
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a, hv[j].x, hv[j].y);
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();

  // epilogue: Ynew[row, state] = alpha*acc + beta*Y[row, state] + delta*X[row, state]
  const int* rm = rowmap + (int64_t)tile * TR;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int row = __ldg(rm + (wn * 4 + j) * 8 + 2 * tt + h);
      if (row < 0) continue;
#pragma unroll
      for (int i = 0; i < MT; ++i) {
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const int state = s_base + (wm * MT + i) * 16 + g + v * 8;
          if (state >= k) continue;
          const int64_t off = (int64_t)row * ld + state;
          float y;
          if constexpr (sizeof(T) == 4) y = __ldg(src + off);
          else y = __bfloat162float(src[off]);
          float o = alpha * acc[i][j][v * 2 + h] + beta * y;
          if (delta != 0.f) {
            float x;
            if constexpr (sizeof(T) == 4) x = xold[off];
            else x = __bfloat162float(xold[off]);
            o = fmaf(delta, x, o);
          }
          if constexpr (sizeof(T) == 4) dst[off] = o;
          else dst[off] = __float2bfloat16_rn(o);
        }
      }
    }
  }
}

uint16_t host_bf16(double v) {
  float f = (float)v;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);   // inf/nan
  const uint32_t rounding = 0x7fffu + ((u >> 16) & 1u);                 // nearest even
  return (uint16_t)((u + rounding) >> 16);
}

}  // namespace

ttg_status build_tiles(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                       const double* hv, int32_t nproj, const int64_t* cp, const int32_t* cc,
                       const double* cv, const int32_t* dims) {
  // rows of each tile
  std::vector<int32_t> rowmap;
  int64_t ntiles;
  if (dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0 &&
      (int64_t)dims[0] * dims[1] * dims[2] == n) {
    const int rx = dims[0], ry = dims[1], rz = dims[2];
    const int bx = (rx + 3) / 4, by = (ry + 3) / 4, bz = (rz + 3) / 4;
    ntiles = (int64_t)bx * by * bz;
    rowmap.assign(ntiles * TR, -1);
    for (int tz = 0; tz < bz; ++tz)
      for (int ty = 0; ty < by; ++ty)
        for (int tx = 0; tx < bx; ++tx) {
          const int64_t t = tx + (int64_t)bx * (ty + (int64_t)by * tz);
          int slot = 0;
          for (int z = 0; z < 4; ++z)
            for (int y = 0; y < 4; ++y)
              for (int x = 0; x < 4; ++x, ++slot) {
                const int X = 4 * tx + x, Y = 4 * ty + y, Z = 4 * tz + z;
                if (X < rx && Y < ry && Z < rz)
                  rowmap[t * TR + slot] = X + rx * (Y + ry * Z);
              }
        }
  } else {
    ntiles = (n + TR - 1) / TR;
    rowmap.assign(ntiles * TR, -1);
    for (int64_t i = 0; i < n; ++i) rowmap[i] = (int32_t)i;
  }
  // C^T rows: (n + a, C[a, i]) for each basis row i
  std::vector<int64_t> tp(n + 1, 0);
  std::vector<int32_t> tcv;
  std::vector<double> tvv;
  if (nproj > 0) {
    for (int a = 0; a < nproj; ++a)
      for (int64_t e = cp[a]; e < cp[a + 1]; ++e) tp[cc[e] + 1]++;
    for (int64_t i = 0; i < n; ++i) tp[i + 1] += tp[i];
    tcv.resize(tp[n]);
    tvv.resize(tp[n]);
    std::vector<int64_t> f(tp.begin(), tp.end() - 1);
    for (int a = 0; a < nproj; ++a)
      for (int64_t e = cp[a]; e < cp[a + 1]; ++e) {
        tcv[f[cc[e]]] = (int32_t)(n + a);
        tvv[f[cc[e]]] = cv[e];
        f[cc[e]]++;
      }
  }
  // merged sorted column list of a tile
  auto merge = [&](int64_t t, std::vector<int32_t>& cols) {
    cols.clear();
    for (int s = 0; s < TR; ++s) {
      const int32_t r = rowmap[t * TR + s];
      if (r < 0) continue;
      cols.insert(cols.end(), hc + hp[r], hc + hp[r + 1]);
      if (nproj > 0) cols.insert(cols.end(), tcv.begin() + tp[r], tcv.begin() + tp[r + 1]);
    }
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
  };
  std::vector<int64_t> tptr(ntiles + 1, 0);
#pragma omp parallel
  {
    std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 4)
    for (int64_t t = 0; t < ntiles; ++t) {
      merge(t, cols);
      tptr[t + 1] = ((int64_t)cols.size() + CS - 1) / CS * CS;
    }
  }
  for (int64_t t = 0; t < ntiles; ++t) tptr[t + 1] += tptr[t];
  const int64_t slots = tptr[ntiles];
  const int64_t nchunk = slots / CS;
  std::vector<int32_t> tcol(std::max<int64_t>(slots, CS), 0);
  // per chunk and n-tile: 32 lanes x 4 values
  std::vector<float> v32((size_t)std::max<int64_t>(nchunk, 1) * 8 * 32 * 4, 0.f);
  std::vector<uint16_t> v16((size_t)std::max<int64_t>(nchunk, 1) * 8 * 32 * 4, 0);
  // for value updates: per H_loc entry, the lane base ((chunk*8 + n-tile)*32 + 4g)
  // of its fragment and its slot within the 16-slot chunk
  const bool keep = op->keep_pattern;
  std::vector<int32_t> tbase(keep ? hp[n] : 0);
  std::vector<uint8_t> tslot(keep ? hp[n] : 0);
  if (keep && nchunk * 8 * 32 >= INT32_MAX) return TTG_BAD_ARG;
#pragma omp parallel
  {
    std::vector<int32_t> cols;
    std::vector<double> dense;   // [slot][64]
#pragma omp for schedule(dynamic, 4)
    for (int64_t t = 0; t < ntiles; ++t) {
      merge(t, cols);
      const int64_t ns = tptr[t + 1] - tptr[t];
      dense.assign((size_t)ns * TR, 0.0);
      for (int64_t s = 0; s < ns; ++s)
        tcol[tptr[t] + s] = cols.empty() ? 0 : cols[std::min<int64_t>(s, (int64_t)cols.size() - 1)];
      for (int s = 0; s < TR; ++s) {
        const int32_t r = rowmap[t * TR + s];
        if (r < 0) continue;
        for (int pass = 0; pass < 2; ++pass) {
          const int32_t* C = pass == 0 ? hc + hp[r] : tcv.data() + (nproj ? tp[r] : 0);
          const double* V = pass == 0 ? hv + hp[r] : tvv.data() + (nproj ? tp[r] : 0);
          const int64_t cnt = pass == 0 ? hp[r + 1] - hp[r] : (nproj ? tp[r + 1] - tp[r] : 0);
          for (int64_t e = 0; e < cnt; ++e) {
            const int64_t slot = std::lower_bound(cols.begin(), cols.end(), C[e]) - cols.begin();
            dense[(size_t)slot * TR + s] = V[e];
            if (keep && pass == 0) {
              const int64_t ge = hp[r] + e;
              const int64_t chunk = tptr[t] / CS + slot / CS;
              tbase[ge] = (int32_t)((chunk * 8 + s / 8) * 32 + 4 * (s % 8));
              tslot[ge] = (uint8_t)(slot % CS);
            }
          }
        }
      }
      const int64_t c0 = tptr[t] / CS;
      for (int64_t c = 0; c < ns / CS; ++c)
        for (int nt = 0; nt < 8; ++nt)
          for (int l = 0; l < 32; ++l) {
            const int gg = l >> 2, q = l & 3;
            const int row = nt * 8 + gg;
            const size_t o = (((size_t)(c0 + c) * 8 + nt) * 32 + l) * 4;
            auto H = [&](int sl) { return dense[(size_t)(c * CS + sl) * TR + row]; };
            // TF32 m16n8k8 B fragment: (k=q, n=g), (k=q+4, n=g), for k8 steps 0 and 1
            v32[o + 0] = (float)H(q);
            v32[o + 1] = (float)H(q + 4);
            v32[o + 2] = (float)H(8 + q);
            v32[o + 3] = (float)H(8 + q + 4);
            // BF16 m16n8k16 B fragment: (k=2q,2q+1; n=g), (k=2q+8,2q+9; n=g)
            v16[o + 0] = host_bf16(H(2 * q));
            v16[o + 1] = host_bf16(H(2 * q + 1));
            v16[o + 2] = host_bf16(H(2 * q + 8));
            v16[o + 3] = host_bf16(H(2 * q + 9));
          }
    }
  }
  TileOp& T = op->tiles;
  T.n_tiles = ntiles;
  T.slots = slots;
  TTG_TRY(T.tptr.alloc((ntiles + 1) * sizeof(int64_t)));
  TTG_TRY(T.tcol.alloc(tcol.size() * sizeof(int32_t)));
  TTG_TRY(T.rowmap.alloc(rowmap.size() * sizeof(int32_t)));
  TTG_TRY(T.v32.alloc(v32.size() * sizeof(float)));
  TTG_TRY(T.v16.alloc(v16.size() * sizeof(uint16_t)));
  TTG_CUDA_TRY(cudaMemcpyAsync(T.tptr.p, tptr.data(), T.tptr.bytes, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(T.tcol.p, tcol.data(), T.tcol.bytes, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(T.rowmap.p, rowmap.data(), T.rowmap.bytes, cudaMemcpyHostToDevice,
                               op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(T.v32.p, v32.data(), T.v32.bytes, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(T.v16.p, v16.data(), T.v16.bytes, cudaMemcpyHostToDevice, op->stream));
  if (keep && hp[n] > 0) {
    Pattern& P = op->pattern;
    TTG_TRY(P.tile_base.alloc(hp[n] * sizeof(int32_t)));
    TTG_TRY(P.tile_slot.alloc(hp[n]));
    TTG_CUDA_TRY(cudaMemcpyAsync(P.tile_base.p, tbase.data(), hp[n] * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, op->stream));
    TTG_CUDA_TRY(cudaMemcpyAsync(P.tile_slot.p, tslot.data(), hp[n], cudaMemcpyHostToDevice,
                                 op->stream));
    op->device_bytes += P.tile_base.bytes + P.tile_slot.bytes;
  }
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  op->device_bytes += T.tptr.bytes + T.tcol.bytes + T.rowmap.bytes + T.v32.bytes + T.v16.bytes;
  return TTG_OK;
}

template <typename T, int MT>
static ttg_status launch_tc_t(ttg_op* op, const void* hval, const void* src, const void* xold,
                              void* dst, int k, double alpha, double beta, double delta) {
  constexpr int KS = 32 * MT;
  dim3 grid((unsigned)op->tiles.n_tiles, (unsigned)((k + KS - 1) / KS));
  TTG_TRY(kt_begin(op, std::is_same<T, float>::value ? TTG_KT_TC_FP32 : TTG_KT_TC_BF16));
  k_cheb_tc<T, MT><<<grid, 128, 0, op->stream>>>(
      op->tiles.tptr.as<int64_t>(), op->tiles.tcol.as<int>(), op->tiles.rowmap.as<int>(),
      reinterpret_cast<const typename TcTraits<T>::HV*>(hval), reinterpret_cast<const T*>(src),
      reinterpret_cast<const T*>(xold), reinterpret_cast<T*>(dst), k, op->ld, (float)alpha,
      (float)beta, (float)delta); TTG_COUNT();
  TTG_LAUNCHED(op);
  TTG_TRY(kt_end(op));
  return TTG_OK;
}

bool tc_supported(const ttg_op* op, int prec, int k) {
  if (op->tiles.n_tiles == 0 || op->tc_disabled) return false;
  if (prec == TTG_PREC_FP32) return k % 4 == 0;
  if (prec == TTG_PREC_BF16) return k % 8 == 0;
  return false;
}

ttg_status launch_cheb_tc(ttg_op* op, int prec, const void* src, const void* xold, void* dst,
                          int k, double alpha, double beta, double delta) {
  const int mt = std::min(5, (k + 31) / 32);
  if (prec == TTG_PREC_FP32) {
    const void* hv = op->tiles.v32.p;
    switch (mt) {
      case 1: return launch_tc_t<float, 1>(op, hv, src, xold, dst, k, alpha, beta, delta);
      case 2: return launch_tc_t<float, 2>(op, hv, src, xold, dst, k, alpha, beta, delta);
      case 3: return launch_tc_t<float, 3>(op, hv, src, xold, dst, k, alpha, beta, delta);
      case 4: return launch_tc_t<float, 4>(op, hv, src, xold, dst, k, alpha, beta, delta);
      default: return launch_tc_t<float, 5>(op, hv, src, xold, dst, k, alpha, beta, delta);
    }
  }
  const void* hv = op->tiles.v16.p;
  switch (mt) {
    case 1: return launch_tc_t<__nv_bfloat16, 1>(op, hv, src, xold, dst, k, alpha, beta, delta);
    case 2: return launch_tc_t<__nv_bfloat16, 2>(op, hv, src, xold, dst, k, alpha, beta, delta);
    case 3: return launch_tc_t<__nv_bfloat16, 3>(op, hv, src, xold, dst, k, alpha, beta, delta);
    case 4: return launch_tc_t<__nv_bfloat16, 4>(op, hv, src, xold, dst, k, alpha, beta, delta);
    default: return launch_tc_t<__nv_bfloat16, 5>(op, hv, src, xold, dst, k, alpha, beta, delta);
  }
}

}  // namespace ttg
