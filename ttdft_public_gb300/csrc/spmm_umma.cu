// FP32-accurate filter degree on the fifth-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory), for the FP32 degrees of the
// Chebyshev filter (ChebyShevFilter.cc:97-170: Ynew = alpha (H Y) + beta Y +
// delta X).
//
// Tiles.  128 rows per tile (a 4 x 4 x 8 block of the Tucker index, or 128
// consecutive rows without Tucker ranks); the tile's sorted column union is
// padded to chunks of 16 slots.  A chunk is one MMA step: M = 128 rows,
// N = k states, K = 16 slots.
//
// Precision.  Every FP32 value v is split into three BF16 terms
// v = v0 + v1 + v2 (|v1| <= 2^-9 |v|, |v2| <= 2^-18 |v|).  The product H Y
// is accumulated in FP32 from the six term products of order <= 2
// (v0w0, v0w1, v1w0, v1w1, v0w2, v2w0); the dropped ones are below 2^-26 of
// the product, so the result carries FP32 accuracy at BF16 MMA rates.
//
// Data movement per chunk.
//  - H: the three BF16 planes of the chunk (128 x 16 values each, already in
//    the canonical K-major no-swizzle layout of the MMA operand) are one
//    contiguous 12 KB block, copied by one bulk asynchronous copy (TMA)
//    that completes on an mbarrier.
//  - Y: the 16 source rows are gathered from three BF16 planes of the block
//    (written by k_split3 before the launch) into the canonical MN-major
//    layout with 16-byte cp.async copies.
// Warp-specialised pipeline: up to nine producer warps take whole chunks in
// turn and fill their stage (the H block by TMA; the gathered rows by cp.async,
// which the warp waits for and fences for the async proxy before it signals
// the stage's mbarrier); one thread of warp 1 issues the six MMAs of a chunk
// as soon as the stage is full and commits them to the stage's "done"
// mbarrier, after which the stage is refilled.  As many stages as fit in
// shared memory (8 for 160 states, one CTA per SM).  The epilogue reads the
// accumulator from tensor memory (one warp per 32 rows) and applies the
// recurrence in FP32.
// Every mbarrier wait is bounded; a wait that runs out sets an error word.

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ttg_internal.cuh"

namespace ttg {
namespace {

constexpr int UR = 128;                       // rows per tile (MMA M)
constexpr int UK = 16;                        // slots per chunk (MMA K)
constexpr int PLANE_ELEMS = UR * UK;          // 2048 BF16 = 4096 bytes
constexpr int CHUNK_ELEMS = 3 * PLANE_ELEMS;  // three planes
constexpr int CHUNK_BYTES = 2 * CHUNK_ELEMS;  // 12288
constexpr int kMaxStages = 8;                // pipeline depth: as many as fit in shared memory
constexpr int kSmemBudget = 227 * 1024 - 1024;
constexpr int kThreads = 320;                // 10 warps
constexpr int kProducerWarps = 9;             // every warp but warp 1 loads (at most nst of them)
constexpr int kMmaWarp = 1;                   // warp 1 issues the MMAs
constexpr int kMaxWait = 1 << 20;
constexpr int kColAhead = 4;                  // chunks per warp whose column indices are loaded ahead

// Canonical no-swizzle layouts (8 x 16-byte core matrices, 128 bytes each):
// core matrices 128 bytes apart along K and 256 bytes apart along M / N.
__host__ __device__ inline int a_elem(int m, int s) {
  return (m >> 3) * 128 + (s >> 3) * 64 + (m & 7) * 8 + (s & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;        // leading byte offset: next core matrix along K
  d |= (uint64_t)(256 >> 4) << 32;        // stride byte offset: next core matrix along M/N
  d |= (uint64_t)1 << 46;                 // descriptor version
  return d;                               // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: BF16 x BF16 -> FP32, A K-major, B MN-major
__device__ __forceinline__ uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 16) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (int i = 0; i < kMaxWait; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(kThreads) k_cheb_umma(
    const int64_t* __restrict__ tptr, const int* __restrict__ tcol, const int* __restrict__ rowmap,
    const int* __restrict__ order, const __nv_bfloat16* __restrict__ hpl, const __nv_bfloat16* __restrict__ xpl,
    int64_t pstride, int ps, const float* __restrict__ src, const float* xold, float* dst,
    int k, int64_t ld, float alpha, float beta, float delta,
    uint32_t tmem_cols, int nst, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kMaxStages];
  __shared__ __align__(8) uint64_t mdone[kMaxStages];
  __shared__ __align__(8) uint64_t accf;     // all MMAs of the tile done (one phase)
  __shared__ uint32_t tmem_slot;
  // tiles in decreasing chunk count, so the longest start first and the short
  // ones fill the tail of the launch
  const int tile = __ldg(order + blockIdx.x), tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int stage_bytes = CHUNK_BYTES + 96 * k;          // H planes + 3 block planes
  const int64_t c_first = tptr[tile] / UK;
  const int nch = (int)((tptr[tile + 1] - tptr[tile]) / UK);
  const int ngrp = k >> 3;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_slot)), "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 2);                    // the owning warp: H copy's expect_tx + rows fenced
      mbar_init(&mdone[s], 1);                   // one tcgen05.commit
    }
    mbar_init(&accf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  bool ok = true;

  if (warp != kMmaWarp) {
    // producers: warps 0, 2, 3, ... (pw = 0 .. np-1) take whole chunks in turn,
    // chunk c to warp c % np.  Chunk c goes into stage c % nst once the MMAs of
    // chunk c - nst have read it; np <= nst keeps every waiter within one phase
    // of the stage's "done" barrier (a warp's previous chunk c - np waited for
    // chunk c - np - nst >= c - 2 nst).  The owning warp arrives on the stage's
    // "full" barrier once its row copies have landed and are fenced; the H
    // block completes by byte count.  A warp waits for its own copies only:
    // the np warps fill np stages at once.
    const int np = min(kProducerWarps, nst);
    const int pw = warp == 0 ? 0 : warp - 1;
    if (pw < np) {
      const int lsl = lane & 15, lhalf = lane >> 4;
      // lane = slot (16) x half (2) of a 32-byte sector: one instruction writes
      // 512 contiguous bytes of shared memory
      const __nv_bfloat16* xl = xpl + 8 * lhalf;
      const uint32_t dl = (uint32_t)(lhalf * 256 + lsl * 16);
      const int* colp = tcol + c_first * UK + lsl;
      // column indices of this warp's next kColAhead chunks live in registers
      int cur[kColAhead], nxt[kColAhead];
#pragma unroll
      for (int j = 0; j < kColAhead; ++j) {
        const int c = pw + j * np;
        cur[j] = c < nch ? __ldg(colp + (int64_t)c * UK) : 0;
      }
      for (int c0 = pw; c0 < nch; c0 += kColAhead * np) {
#pragma unroll
        for (int j = 0; j < kColAhead; ++j) {
          const int c = c0 + (kColAhead + j) * np;
          nxt[j] = c < nch ? __ldg(colp + (int64_t)c * UK) : 0;
        }
#pragma unroll
        for (int j = 0; j < kColAhead; ++j) {
          const int c = c0 + j * np;
          if (c >= nch) break;
          const int s = c % nst;
          if (c >= nst) ok &= mbar_wait(&mdone[s], ((c / nst) - 1) & 1);
          unsigned char* st = smem + s * stage_bytes;
          if (lane == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         ::"r"(smem_u32(&full[s])), "r"(CHUNK_BYTES) : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_u32(st)), "l"(hpl + (c_first + c) * CHUNK_ELEMS), "r"(CHUNK_BYTES),
                "r"(smem_u32(&full[s]))
                : "memory");
          }
          const __nv_bfloat16* xs = xl + (int64_t)cur[j] * ps;
          const uint32_t d0 = smem_u32(st + CHUNK_BYTES) + dl;
#pragma unroll
          for (int pl = 0; pl < 3; ++pl)
            for (int g = 0; g < ngrp; g += 2)   // ngrp = k / 8 is even
              asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                           ::"r"(d0 + (uint32_t)(pl * 32 * k + g * 256)), "l"(xs + pl * pstride + 8 * g)
                           : "memory");
          // the rows were written through the generic proxy: each thread waits
          // for its own copies and fences them for the tensor core's
          // (async-proxy) reads before the warp signals the stage
          cp_async_commit();
          cp_async_wait<0>();
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full[s]))
                         : "memory");
        }
#pragma unroll
        for (int j = 0; j < kColAhead; ++j) cur[j] = nxt[j];
      }
      cp_async_wait<0>();
    }
  } else if (lane == 0) {
    // MMA issuer: six MMAs per chunk (term pairs, smallest products first)
    const uint32_t idesc = instr_desc(UR, k);
    const int pa[6] = {1, 0, 2, 0, 1, 0};
    const int pb[6] = {1, 2, 0, 1, 0, 0};
    for (int c = 0; c < nch; ++c) {
      const int s = c % nst;
      ok &= mbar_wait(&full[s], (c / nst) & 1);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(smem + s * stage_bytes);
      const uint32_t b0 = a0 + CHUNK_BYTES;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const uint64_t da = smem_desc(a0 + pa[q] * (2 * PLANE_ELEMS));
        const uint64_t db = smem_desc(b0 + pb[q] * (32 * k));
        const uint32_t acc = (c > 0 || q > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
            ::"r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(smem_u32(&mdone[s]))
          : "memory");
    }
    if (nch > 0)
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(smem_u32(&accf))
          : "memory");
  }
  __syncwarp();
  // all MMAs done.  A barrier of its own, used for one phase: a thread may
  // get here long before the last chunk's stage barrier has passed the phase
  // before its last one, where a parity wait on it would pass early.
  if (nch > 0) ok &= mbar_wait(&accf, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue (warps 0-3, one per 32 TMEM lanes): row = warp*32 + lane of the
  // tile, 16 states per TMEM load
  if (warp < 4) {
  const int row = __ldg(rowmap + (int64_t)tile * UR + warp * 32 + lane);
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  for (int c0 = 0; c0 < k; c0 += 16) {
    uint32_t v[16];
    if (nch > 0) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(lane_base + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = 0u;
    }
    if (row >= 0) {
      const int64_t off = (int64_t)row * ld + c0;
#pragma unroll
      for (int j = 0; j < 16; j += 4) {
        const float4 y = *reinterpret_cast<const float4*>(src + off + j);
        float4 o;
        o.x = alpha * __uint_as_float(v[j]) + beta * y.x;
        o.y = alpha * __uint_as_float(v[j + 1]) + beta * y.y;
        o.z = alpha * __uint_as_float(v[j + 2]) + beta * y.z;
        o.w = alpha * __uint_as_float(v[j + 3]) + beta * y.w;
        if (delta != 0.f) {
          const float4 x = *reinterpret_cast<const float4*>(xold + off + j);
          o.x = fmaf(delta, x.x, o.x);
          o.y = fmaf(delta, x.y, o.y);
          o.z = fmaf(delta, x.z, o.z);
          o.w = fmaf(delta, x.w, o.w);
        }
        *reinterpret_cast<float4*>(dst + off + j) = o;
      }
    }
  }
  }
  if (!ok) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
}

// Three BF16 terms of each FP32 entry of rows [0, rows) of a block (row
// stride ld), into planes of row stride ps (states k..ps-1 zero).
__global__ void k_split3(const float* __restrict__ src, int64_t rows, int k, int64_t ld,
                         __nv_bfloat16* __restrict__ pl, int ps, int64_t pstride) {
  const int64_t total = rows * ps;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / ps;
    const int c = (int)(i - r * ps);
    const float v = c < k ? src[r * ld + c] : 0.f;
    const __nv_bfloat16 h0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(h0);
    const __nv_bfloat16 h1 = __float2bfloat16_rn(r1);
    const __nv_bfloat16 h2 = __float2bfloat16_rn(r1 - __bfloat162float(h1));
    pl[i] = h0;
    pl[pstride + i] = h1;
    pl[2 * pstride + i] = h2;
  }
}

uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);
  const uint32_t rounding = 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)((u + rounding) >> 16);
}

float bf16_float(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// v = t0 + t1 + t2 as on the device (float steps from the value rounded to FP32
// first, residuals in double).
void split3_host(double v, uint16_t* t) {
  t[0] = bf16_bits((float)v);
  const double r1 = v - bf16_float(t[0]);
  t[1] = bf16_bits((float)r1);
  t[2] = bf16_bits((float)(r1 - bf16_float(t[1])));
}

int umma_disabled_by_env() {
  const char* e = getenv("TTG_DISABLE_UMMA");
  return e && e[0] == '1';
}

}  // namespace

ttg_status build_umma_tiles(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                            const double* hv, int32_t nproj, const int64_t* cp, const int32_t* cc,
                            const double* cv, const int32_t* dims) {
  if (umma_disabled_by_env()) return TTG_OK;
  std::vector<int32_t> rowmap;
  int64_t ntiles;
  if (dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0 &&
      (int64_t)dims[0] * dims[1] * dims[2] == n) {
    const int rx = dims[0], ry = dims[1], rz = dims[2];
    const int bx = (rx + 3) / 4, by = (ry + 3) / 4, bz = (rz + 7) / 8;
    ntiles = (int64_t)bx * by * bz;
    rowmap.assign(ntiles * UR, -1);
    for (int tz = 0; tz < bz; ++tz)
      for (int ty = 0; ty < by; ++ty)
        for (int tx = 0; tx < bx; ++tx) {
          const int64_t t = tx + (int64_t)bx * (ty + (int64_t)by * tz);
          int slot = 0;
          for (int z = 0; z < 8; ++z)
            for (int y = 0; y < 4; ++y)
              for (int x = 0; x < 4; ++x, ++slot) {
                const int X = 4 * tx + x, Y = 4 * ty + y, Z = 8 * tz + z;
                if (X < rx && Y < ry && Z < rz) rowmap[t * UR + slot] = X + rx * (Y + ry * Z);
              }
        }
  } else {
    ntiles = (n + UR - 1) / UR;
    rowmap.assign(ntiles * UR, -1);
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
  auto merge = [&](int64_t t, std::vector<int32_t>& cols) {
    cols.clear();
    for (int s = 0; s < UR; ++s) {
      const int32_t r = rowmap[t * UR + s];
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
      tptr[t + 1] = ((int64_t)cols.size() + UK - 1) / UK * UK;
    }
  }
  std::vector<int32_t> order(ntiles);
  for (int64_t t = 0; t < ntiles; ++t) order[t] = (int32_t)t;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return tptr[a + 1] > tptr[b + 1]; });
  for (int64_t t = 0; t < ntiles; ++t) tptr[t + 1] += tptr[t];
  const int64_t slots = tptr[ntiles];
  const int64_t nchunk = slots / UK;
  const bool keep = op->keep_pattern;
  if (nchunk * (int64_t)CHUNK_ELEMS >= INT32_MAX && keep) return TTG_OK;   // no map possible
  std::vector<int32_t> tcol(std::max<int64_t>(slots, UK), 0);
  std::vector<uint16_t> hpl((size_t)std::max<int64_t>(nchunk, 1) * CHUNK_ELEMS, 0);
  std::vector<int32_t> pos(keep ? hp[n] : 0);
#pragma omp parallel
  {
    std::vector<int32_t> cols;
#pragma omp for schedule(dynamic, 4)
    for (int64_t t = 0; t < ntiles; ++t) {
      merge(t, cols);
      const int64_t ns = tptr[t + 1] - tptr[t];
      for (int64_t s = 0; s < ns; ++s)
        tcol[tptr[t] + s] = cols.empty() ? 0 : cols[std::min<int64_t>(s, (int64_t)cols.size() - 1)];
      const int64_t c0 = tptr[t] / UK;
      for (int m = 0; m < UR; ++m) {
        const int32_t r = rowmap[t * UR + m];
        if (r < 0) continue;
        for (int pass = 0; pass < 2; ++pass) {
          const int32_t* C = pass == 0 ? hc + hp[r] : tcv.data() + (nproj ? tp[r] : 0);
          const double* V = pass == 0 ? hv + hp[r] : tvv.data() + (nproj ? tp[r] : 0);
          const int64_t cnt = pass == 0 ? hp[r + 1] - hp[r] : (nproj ? tp[r + 1] - tp[r] : 0);
          for (int64_t e = 0; e < cnt; ++e) {
            const int64_t slot = std::lower_bound(cols.begin(), cols.end(), C[e]) - cols.begin();
            const int64_t base = (c0 + slot / UK) * CHUNK_ELEMS + a_elem(m, (int)(slot % UK));
            uint16_t tt[3];
            split3_host(V[e], tt);
            for (int p = 0; p < 3; ++p) hpl[base + p * PLANE_ELEMS] = tt[p];
            if (keep && pass == 0) pos[hp[r] + e] = (int32_t)base;
          }
        }
      }
    }
  }
  UmmaOp& U = op->umma;
  U.n_tiles = ntiles;
  U.slots = slots;
  TTG_TRY(U.tptr.alloc((ntiles + 1) * sizeof(int64_t)));
  TTG_TRY(U.tcol.alloc(tcol.size() * sizeof(int32_t)));
  TTG_TRY(U.rowmap.alloc(rowmap.size() * sizeof(int32_t)));
  TTG_TRY(U.order.alloc(order.size() * sizeof(int32_t)));
  TTG_TRY(U.hpl.alloc(hpl.size() * sizeof(uint16_t)));
  TTG_TRY(U.err.alloc(sizeof(int)));
  TTG_CUDA_TRY(cudaMemcpyAsync(U.tptr.p, tptr.data(), U.tptr.bytes, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(U.tcol.p, tcol.data(), U.tcol.bytes, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(U.rowmap.p, rowmap.data(), U.rowmap.bytes, cudaMemcpyHostToDevice,
                               op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(U.order.p, order.data(), U.order.bytes, cudaMemcpyHostToDevice,
                               op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(U.hpl.p, hpl.data(), U.hpl.bytes, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaMemsetAsync(U.err.p, 0, sizeof(int), op->stream));
  if (keep && hp[n] > 0) {
    TTG_TRY(op->pattern.umma_pos.alloc(hp[n] * sizeof(int32_t)));
    TTG_CUDA_TRY(cudaMemcpyAsync(op->pattern.umma_pos.p, pos.data(), hp[n] * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, op->stream));
    op->device_bytes += op->pattern.umma_pos.bytes;
  }
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  op->device_bytes += U.tptr.bytes + U.tcol.bytes + U.rowmap.bytes + U.order.bytes + U.hpl.bytes;
  return TTG_OK;
}

bool umma_supported(const ttg_op* op, int prec, int k) {
  return prec == TTG_PREC_FP32 && op->umma.n_tiles > 0 && !op->tc_disabled && k >= 16 &&
         k <= 256 && k % 16 == 0 && k <= op->ld;
}

ttg_status launch_cheb_umma(ttg_op* op, const void* src, const void* xold, void* dst, int k,
                            double alpha, double beta, double delta) {
  UmmaOp& U = op->umma;
  const int ps = k;                                  // multiple of 16
  const int64_t rows = op->n + op->nproj;
  const int64_t pstride = rows * ps;
  const size_t need = (size_t)3 * pstride * sizeof(uint16_t);
  if (U.xpl.bytes < need) {
    TTG_TRY(U.xpl.alloc(need));
    op->device_bytes += (int64_t)need;
  }
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_cheb_umma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kSmemBudget);
  });
  if (attr_err != cudaSuccess) return TTG_CUDA_ERR;
  const int grid_s = (int)std::min<int64_t>((rows * ps + 255) / 256, 152 * 16);
  k_split3<<<grid_s, 256, 0, op->stream>>>(reinterpret_cast<const float*>(src), rows, k, op->ld,
                                           U.xpl.as<__nv_bfloat16>(), ps, pstride); TTG_COUNT();
  TTG_LAUNCHED(op);
  uint32_t cols = 32;
  while ((int)cols < k) cols <<= 1;
  const int stage_bytes = CHUNK_BYTES + 96 * k;
  const int nst = std::min(kMaxStages, kSmemBudget / stage_bytes);
  if (nst < 3) return TTG_BAD_ARG;
  const size_t smem = (size_t)nst * stage_bytes;
  k_cheb_umma<<<(unsigned)U.n_tiles, kThreads, smem, op->stream>>>(
      U.tptr.as<int64_t>(), U.tcol.as<int>(), U.rowmap.as<int>(), U.order.as<int>(),
      U.hpl.as<__nv_bfloat16>(),
      U.xpl.as<__nv_bfloat16>(), pstride, ps, reinterpret_cast<const float*>(src),
      reinterpret_cast<const float*>(xold), reinterpret_cast<float*>(dst), k, op->ld,
      (float)alpha, (float)beta, (float)delta, cols, nst, U.err.as<int>()); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

ttg_status umma_check_error(ttg_op* op) {
  if (op->umma.n_tiles == 0) return TTG_OK;
  int e = 0;
  TTG_CUDA_TRY(cudaMemcpyAsync(&e, op->umma.err.p, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  if (e) {
    TTG_CUDA_TRY(cudaMemsetAsync(op->umma.err.p, 0, sizeof(int), op->stream));
    return TTG_TIMEOUT;
  }
  return TTG_OK;
}

}  // namespace ttg
