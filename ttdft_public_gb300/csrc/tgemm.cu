// Dense contractions on the fifth-generation tensor cores (tcgen05.mma with
// the accumulator in tensor memory), FP32-accurate and free of accumulation
// rounding.
//
// C(m, n) = sum_k A(m, k) B(n, k) for FP32 operands stored K-contiguous
// (row-major, one row per m or n), optionally batched over z, with the K
// range cut into G groups (the Hartree expansion's terms, or the density's
// states) whose results the epilogue combines in double-FP32.
//
// Arithmetic (an Ozaki-type error-free split).  The tensor cores' FP32
// accumulation does not round to nearest: measured on the Hartree
// contraction with FP32 operands split into three BF16 terms, the products
// accumulated in one FP32 accumulator kept only ~7e-7 relative accuracy over
// a few dozen additions, as if each addition were truncated toward zero.
// Instead, every operand value v of a group (or batch) with max |v| < 2^e is
// cut into three integer slices on a common grid,
//   v 2^(8-e) = a0 + a1 2^-8 + a2 2^-16 + O(2^-17),  a_p integers, |a_p| <= 256,
// which BF16 holds exactly.  Products of slices are exact integers; the sums
// of one level L = p + q (a0b0; a0b1 + a1b0; a0b2 + a1b1 + a2b0; a1b2 + a2b1)
// stay below 2^24 for a group of up to 192 K values, so each level
// accumulates in its own tensor-memory accumulator without rounding
// (integer-valued operands come out exact); only a2b2, 2^-32 of the leading
// product, is left out.  The epilogue adds S0 + S1 2^-8 + S2 2^-16 + S3 2^-24
// with error-free two-sums (the levels can cancel), scales by
// 2^(eA + eB - 16) and sums the groups in double-FP32: the result carries the
// operands' FP32 quantisation (2^-25 of each group's largest value) and
// nothing else.  The group maxima come from the kernels that write the
// operands (atomicMax on |v|).
//
// Data movement (one CTA per SM, persistent over output tiles of 128 x 48):
//  - warp 0, one thread: TMA tiled loads (cp.async.bulk.tensor) of the FP32
//    tiles A[128 rows][16] and B[48 rows][16] of one K-chunk into a raw
//    ring; rows and K beyond the tensor's extent are filled with zeros;
//  - warp 3, one thread: waits for the raw stages' copies in order and
//    publishes the count of landed chunks.  The converter warps take chunks
//    round-robin, so one polling a stage's barrier itself could meet it a
//    phase early (the previous chunk of that stage, another warp's, still in
//    flight) and read the stage's previous-but-one completion as its own;
//  - warps 4-9, whole chunks in turn: slice the chunk's 176 rows into three
//    BF16 planes each, written in the canonical K-major layout of the MMA
//    operands (8-row x 16-byte core matrices), fence them for the async
//    proxy, arrive;
//  - warp 2, one thread: waits for each chunk's slices (and, at the start of
//    a group, for the epilogue to have emptied the accumulators the group
//    will use) and publishes the count of ready chunks;
//  - warp 1, one thread: eight MMAs (M128 N48 K16) per chunk into the four
//    level accumulators of one of two buffers (double-buffered across
//    groups), a commit per chunk to free the slice stage and per group to
//    hand the buffer to the epilogue;
//  - warps 10-17 (two per 32 TMEM lanes, 24 columns each): combine the levels
//    and store (one group: FP32, with the output's per-batch max |v| for the
//    next contraction) or add into hi/lo sums kept in tensor memory after the
//    two buffers, stored as FP64 after the last group.
// Every wait is bounded; a wait that runs out sets the error word and an
// abort flag that stops every role from issuing further work.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "ttg_internal.cuh"
#include "tgemm.cuh"
#include "tc_common.cuh"

namespace ttg {
namespace {

using namespace tc;

constexpr int TG_M = 128;                         // rows of an A tile (MMA M)
constexpr int TG_N = 48;                          // rows of a B tile (MMA N)
constexpr int TG_K = 16;                          // K per chunk (one MMA)
constexpr int kRawA = TG_M * TG_K * 4;            // 8 KB FP32
constexpr int kRawB = TG_N * TG_K * 4;            // 3 KB FP32
constexpr int kRawStage = kRawA + kRawB;          // 11 KB (a multiple of 1 KB: TMA destinations)
constexpr int kPlaneA = TG_M * TG_K * 2;          // 4 KB: one BF16 slice plane of A
constexpr int kPlaneB = TG_N * TG_K * 2;          // 1.5 KB
constexpr int kSplitStage = 3 * kPlaneA + 3 * kPlaneB;   // 16.5 KB
constexpr int kRawStages = 8;
constexpr int kSplitStages = 7;
constexpr int kSmem = kRawStages * kRawStage + kSplitStages * kSplitStage + 1024;
constexpr int kConvWarp0 = 4, kConvWarps = 6;     // whole chunks in turn (<= kSplitStages)
constexpr int kRows = TG_M + TG_N;                // rows a converter warp slices per chunk
constexpr int kEpiWarp0 = 10, kEpiWarps = 8;      // two warps per 32 TMEM lanes
constexpr int kThreads = (kEpiWarp0 + kEpiWarps) * 32;   // 576
constexpr int kBufCols = 4 * TG_N;                // four level accumulators per buffer
constexpr uint32_t kTmemCols = 512;               // 2 buffers (384) + hi, lo (96)



// kind::f16: BF16 x BF16 -> FP32, A and B K-major, M = 128, N = 48
__device__ __forceinline__ uint32_t idesc_mma() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TG_N >> 3) << 17) |
         ((uint32_t)(TG_M >> 4) << 24);
}








struct TileSched {
  int tiles_m, tiles_n;
  __device__ void at(int64_t t, int& tm, int& tn, int& z) const {
    const int64_t per = (int64_t)tiles_m * tiles_n;
    z = (int)(t / per);
    const int64_t r = t - (int64_t)z * per;
    tm = (int)(r / tiles_n);     // n fastest: CTAs that share an A tile run together
    tn = (int)(r - (int64_t)tm * tiles_n);
  }
};

// exponent e with max |v| < 2^e (0 for an all-zero group)
__device__ __forceinline__ int grid_exp(float amax) {
  int e = 0;
  if (amax > 0.f) frexpf(amax, &e);
  return e;
}

// three integer slices of 8 values on the grid 2^(e-8): v 2^(8-e) = a0 + a1/256 + a2/65536
__device__ __forceinline__ void slice8(const float* v, float sc, uint4& p0, uint4& p1,
                                       uint4& p2) {
  uint32_t w0[4], w1[4], w2[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float a[2], b[2], c[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float x = v[2 * j + h] * sc;          // |x| < 256, exact (power-of-two scale)
      a[h] = rintf(x);
      const float r = (x - a[h]) * 256.f;         // exact, |r| <= 128
      b[h] = rintf(r);
      c[h] = rintf((r - b[h]) * 256.f);
    }
    const __nv_bfloat162 h0 = __floats2bfloat162_rn(a[0], a[1]);   // integers <= 256: exact
    const __nv_bfloat162 h1 = __floats2bfloat162_rn(b[0], b[1]);
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(c[0], c[1]);
    w0[j] = *reinterpret_cast<const uint32_t*>(&h0);
    w1[j] = *reinterpret_cast<const uint32_t*>(&h1);
    w2[j] = *reinterpret_cast<const uint32_t*>(&h2);
  }
  p0 = make_uint4(w0[0], w0[1], w0[2], w0[3]);
  p1 = make_uint4(w1[0], w1[1], w1[2], w1[3]);
  p2 = make_uint4(w2[0], w2[1], w2[2], w2[3]);
}



}  // namespace
}  // namespace ttg

namespace ttg {
namespace {

template <int MODE>
__global__ void __launch_bounds__(kThreads, 1) k_tgemm(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int a3d,
    int b3d, const float* __restrict__ amaxA, const float* __restrict__ amaxB, int M, int N,
    int Z, int G, int kg, TileSched sch, TOut out, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (su32(smem_raw) & 1023)) & 1023);
  unsigned char* raw = smem;                                   // kRawStages x 12 KB
  unsigned char* spl = smem + kRawStages * kRawStage;         // kSplitStages x 18 KB
  __shared__ __align__(8) uint64_t raw_full[kRawStages], raw_empty[kRawStages];
  __shared__ __align__(8) uint64_t spl_full[kSplitStages], spl_empty[kSplitStages];
  __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2];
  __shared__ __align__(8) uint64_t fin;                        // all MMAs issued have completed
  __shared__ uint32_t tmem_slot;
  __shared__ uint32_t ready;                                   // chunks sliced
  __shared__ uint32_t landed;                                  // chunks whose raw copies landed
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (int64_t)sch.tiles_m * sch.tiles_n * Z;
  const int nk = G * kg;                                       // chunks per tile
  int my_tiles = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) ++my_tiles;
  // slice-grid index of the chunk's A and B values
  auto sidx_a = [&](int g, int z) { return MODE == TG_STORE_F32 ? (a3d ? z : 0) : g; };
  auto sidx_b = [&](int g, int z) { return MODE == TG_SUM_F64 ? g : (b3d ? z : 0); };

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(su32(&tmem_slot)), "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 32) {
    for (int s = 0; s < kRawStages; ++s) {
      bar_init(&raw_full[s], 1);
      bar_init(&raw_empty[s], 1);
    }
    for (int s = 0; s < kSplitStages; ++s) {
      bar_init(&spl_full[s], 1);
      bar_init(&spl_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      bar_init(&acc_full[b], 1);
      bar_init(&acc_empty[b], kEpiWarps);
    }
    bar_init(&fin, 1);
    ready = 0;
    landed = 0;
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  volatile int* abrt = &abort_flag;
  bool ok = true;

  if (warp == 0) {
    // ---- TMA producer
    if (lane == 0) {
      int64_t q = 0;
      for (int j = 0; j < my_tiles && ok; ++j) {
        int tm, tn, z;
        sch.at(blockIdx.x + (int64_t)j * gridDim.x, tm, tn, z);
        for (int c = 0; c < nk; ++c, ++q) {
          const int s = (int)(q % kRawStages);
          // TG_SQSUM_F64: group g = c / kg reads batch g of A at chunk c % kg
          const int ka = MODE == TG_SQSUM_F64 ? (c % kg) : c;
          const int za = MODE == TG_SQSUM_F64 ? (c / kg) : z;
          if (q >= kRawStages &&
              !bar_wait(&raw_empty[s], (uint32_t)((q / kRawStages - 1) & 1), abrt, 32)) {
            ok = false;
            break;
          }
          // the stage's previous copy (chunk q - kRawStages) must have landed
          // before this chunk's arrival: otherwise the arrival would fall into
          // that phase.  Holds by construction; checked so that a broken
          // invariant ends the kernel with an error, not with a bad barrier
          if (q >= kRawStages && !bar_test(&raw_full[s], (uint32_t)((q / kRawStages - 1) & 1))) {
            atomicExch(err, 3);
            ok = false;
            *abrt = 1;
            break;
          }
          const uint32_t fb = su32(&raw_full[s]);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb),
                       "r"(kRawStage) : "memory");
          const uint32_t dst = su32(raw + s * kRawStage);
          tma_load(dst, &tmA, ka * TG_K, tm * TG_M, za, a3d != 0, fb);
          tma_load(dst + kRawA, &tmB, ka * TG_K, tn * TG_N, z, b3d != 0, fb);
        }
      }
      // on abort, let the copies already issued land before the CTA exits
      if (!ok)
        for (int64_t r = (q > kRawStages ? q - kRawStages : 0); r < q; ++r)
          bar_drain(&raw_full[r % kRawStages], (uint32_t)((r / kRawStages) & 1));
    }
  } else if (warp >= kConvWarp0 && warp < kConvWarp0 + kConvWarps) {
    // ---- slice whole chunks, chunk q to converter warp q % kConvWarps: the 128 A
    // rows and 48 B rows of a chunk into three integer BF16 planes each
    const int cw = warp - kConvWarp0;
    const int64_t total = (int64_t)my_tiles * nk;
    for (int64_t q = cw; q < total; q += kConvWarps) {
      const int j = (int)(q / nk), c = (int)(q % nk);
      int tm, tn, z;
      sch.at(blockIdx.x + (int64_t)j * gridDim.x, tm, tn, z);
      const int s = (int)(q % kRawStages), s2 = (int)(q % kSplitStages);
      const int g = c / kg;
      const float sca = ldexpf(1.f, 8 - grid_exp(__ldg(amaxA + sidx_a(g, z))));
      const float scb = ldexpf(1.f, 8 - grid_exp(__ldg(amaxB + sidx_b(g, z))));
      bool w = true;
      if (lane == 0) {
        // chunk q has landed (published in order by warp 3)
        w = false;
        for (int i = 0; i < kTcMaxWait; ++i) {
          uint32_t l;
          asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(l) : "r"(su32(&landed))
                       : "memory");
          if (l > (uint32_t)q) { w = true; break; }
          if (*abrt) break;
          __nanosleep(32);
        }
        if (!w) *abrt = 1;
        // the MMAs of chunk q - kSplitStages have read this slice stage
        if (w && q >= kSplitStages)
          w = bar_wait(&spl_empty[s2], (uint32_t)((q / kSplitStages - 1) & 1), abrt, 32);
      }
      w = __shfl_sync(0xffffffffu, w, 0);
      if (!w) { ok = false; break; }
      const unsigned char* src0 = raw + s * kRawStage;
      unsigned char* dst0 = spl + s2 * kSplitStage;
      for (int r = lane; r < kRows; r += 32) {
        const bool isb = r >= TG_M;
        const int row = isb ? r - TG_M : r;
        float v[16];
        const float4* src = reinterpret_cast<const float4*>(src0 + (isb ? kRawA : 0) + row * 64);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 f = src[i];
          v[4 * i] = f.x; v[4 * i + 1] = f.y; v[4 * i + 2] = f.z; v[4 * i + 3] = f.w;
        }
        const int plane = isb ? kPlaneB : kPlaneA;
        unsigned char* dst = dst0 + (isb ? 3 * kPlaneA : 0) + (row >> 3) * 256 + (row & 7) * 16;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint4 p0, p1, p2;
          slice8(v + 8 * h, isb ? scb : sca, p0, p1, p2);
          *reinterpret_cast<uint4*>(dst + h * 128) = p0;
          *reinterpret_cast<uint4*>(dst + plane + h * 128) = p1;
          *reinterpret_cast<uint4*>(dst + 2 * plane + h * 128) = p2;
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        bar_arrive(&raw_empty[s]);
        bar_arrive(&spl_full[s2]);
      }
    }
  } else if (warp == 3) {
    // ---- waits for the raw copies in order; the converters read the count
    if (lane == 0) {
      const int64_t total = (int64_t)my_tiles * nk;
      for (int64_t q = 0; q < total; ++q) {
        if (!bar_wait(&raw_full[q % kRawStages], (uint32_t)((q / kRawStages) & 1), abrt, 32)) {
          ok = false;
          break;
        }
        asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(su32(&landed)),
                     "r"((uint32_t)(q + 1)) : "memory");
      }
    }
  } else if (warp == 2) {
    // ---- waits for slice stages (and emptied accumulators) in order
    if (lane == 0) {
      int64_t q = 0, gg = 0;
      for (int j = 0; j < my_tiles && ok; ++j)
        for (int g = 0; g < G && ok; ++g, ++gg)
          for (int c = 0; c < kg; ++c, ++q) {
            if (c == 0 && gg >= 2 &&
                !bar_wait(&acc_empty[gg & 1], (uint32_t)(((gg >> 1) - 1) & 1), abrt, 32)) {
              ok = false;
              break;
            }
            if (!bar_wait(&spl_full[q % kSplitStages], (uint32_t)((q / kSplitStages) & 1), abrt,
                          16)) {
              ok = false;
              break;
            }
            asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(su32(&ready)),
                         "r"((uint32_t)(q + 1)) : "memory");
          }
    }
  } else if (warp == 1) {
    // ---- MMA issue: six slice products per chunk into three level accumulators
    if (lane == 0) {
      const uint32_t idesc = idesc_mma();
      const uint32_t spl0 = su32(spl);
      int64_t q = 0, gg = 0;
      uint32_t avail = 0;
      // (slice of A, slice of B, level): level 3 first, then 2, 1, 0; the level-4
      // product a2 b2 (2^-32 of the leading one) is left out
      const int ta[8] = {1, 2, 1, 0, 2, 0, 1, 0}, tb[8] = {2, 1, 1, 2, 0, 1, 0, 0};
      const int lv[8] = {3, 3, 2, 2, 2, 1, 1, 0};
      const bool first[8] = {true, false, true, false, false, true, false, true};
      for (int j = 0; j < my_tiles && ok; ++j)
        for (int g = 0; g < G && ok; ++g, ++gg) {
          const uint32_t dbuf = tmem + (uint32_t)((gg & 1) * kBufCols);
          for (int c = 0; c < kg; ++c, ++q) {
            // polling with a short back-off: spinning threads take issue slots
            // from the converter and epilogue warps
            for (int i = 0; i < kTcMaxWait && avail <= (uint32_t)q; ++i) {
              asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(avail)
                           : "r"(su32(&ready)) : "memory");
              if (avail > (uint32_t)q || *abrt) break;
              __nanosleep(16);
            }
            if (avail <= (uint32_t)q) { ok = false; *abrt = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = spl0 + (uint32_t)((q % kSplitStages) * kSplitStage);
#pragma unroll
            for (int p = 0; p < 8; ++p) {
              const uint64_t da = kmajor_desc(base + ta[p] * kPlaneA);
              const uint64_t db = kmajor_desc(base + 3 * kPlaneA + tb[p] * kPlaneB);
              const uint32_t acc = (c > 0 || !first[p]) ? 1u : 0u;
              asm volatile(
                  "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                  ::"r"(dbuf + (uint32_t)(lv[p] * TG_N)), "l"(da), "l"(db), "r"(idesc),
                    "r"(acc));
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                ::"r"(su32(&spl_empty[q % kSplitStages])) : "memory");
          }
          if (!ok) break;
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
              ::"r"(su32(&acc_full[gg & 1])) : "memory");
        }
      // every MMA issued has completed before tensor memory is released
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(su32(&fin)) : "memory");
      bar_drain(&fin, 0);
    }
  } else if (warp >= kEpiWarp0) {
    // ---- epilogue: TMEM lanes 32 (warp & 3) .., columns 24 half .. 24 half + 23
    const int qd = warp & 3, half = (warp - kEpiWarp0) >> 2;
    const int row = qd * 32 + lane;
    const uint32_t lanes = (uint32_t)(qd * 32) << 16;
    int64_t gg = 0;
    for (int j = 0; j < my_tiles && ok; ++j) {
      int tm, tn, z;
      sch.at(blockIdx.x + (int64_t)j * gridDim.x, tm, tn, z);
      const int64_t m = (int64_t)tm * TG_M + row;
      const bool mok = m < M;
      const int64_t base = mok ? (m % out.r1) * out.s1 + (m / out.r1) * out.s2 + z * out.bs : 0;
      const int n0 = tn * TG_N + half * (TG_N / 2);
      // running double-FP32 sums of the groups (TG_SUM_F64, TG_SQSUM_F64) in
      // tensor memory after the two accumulator buffers: hi, then lo
      const uint32_t hcol = tmem + lanes + (uint32_t)(2 * kBufCols + half * (TG_N / 2));
      const uint32_t lcol = hcol + (uint32_t)TG_N;
      float vmax = 0.f;
      bool oob = false;
      for (int g = 0; g < G; ++g, ++gg) {
        if (!bar_wait(&acc_full[gg & 1], (uint32_t)((gg >> 1) & 1), abrt, 64)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // level sums are exact integers on the grid 2^(eA + eB - 16)
        const float scale = ldexpf(1.f, grid_exp(__ldg(amaxA + sidx_a(g, z))) +
                                            grid_exp(__ldg(amaxB + sidx_b(g, z))) - 16);
        const float wg = MODE == TG_SQSUM_F64 ? __ldg(out.w + g) : 0.f;
        const uint32_t acol = tmem + lanes + (uint32_t)((gg & 1) * kBufCols + half * (TG_N / 2));
#pragma unroll
        for (int c0 = 0; c0 < TG_N / 2; c0 += 8) {
          float s0[8], s1[8], s2[8], s3[8];
          tmem_ld8(acol + c0, s0);
          tmem_ld8(acol + TG_N + c0, s1);
          tmem_ld8(acol + 2 * TG_N + c0, s2);
          tmem_ld8(acol + 3 * TG_N + c0, s3);
          // the group's value S0 + S1 2^-8 + S2 2^-16 + S3 2^-24 as an
          // unevaluated pair (vh, vl): the level sums are exact integers and
          // partly cancel, so they are added with error-free two-sums
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float t[3] = {s1[i] * (1.f / 256.f), s2[i] * (1.f / 65536.f),
                                s3[i] * (1.f / 16777216.f)};
            float h = s0[i], l = 0.f;
#pragma unroll
            for (int u = 0; u < 3; ++u) {
              const float h2 = h + t[u];
              const float bv = h2 - h;
              l += (h - (h2 - bv)) + (t[u] - bv);
              h = h2;
            }
            float vh = h * scale, vl = l * scale;
            if constexpr (MODE == TG_STORE_F32) {
              const float v = vh + vl;
              const int64_t n = n0 + c0 + i;
              if (mok && n < N) {
                const int64_t off = base + n * out.cs;
                if ((uint64_t)off < (uint64_t)out.limit) {
                  reinterpret_cast<float*>(out.p)[off] = v;
                  vmax = fmaxf(vmax, fabsf(v));
                } else {
                  oob = true;
                }
              }
            } else {
              if constexpr (MODE == TG_SQSUM_F64) {      // w (vh + vl)^2 to double-FP32
                const float sq = vh * vh;
                const float sqe = fmaf(vh, vh, -sq) + 2.f * vh * vl;
                vh = wg * sq;
                vl = fmaf(wg, sq, -vh) + wg * sqe;
              }
              s0[i] = vh;
              s1[i] = vl;
            }
          }
          if constexpr (MODE != TG_STORE_F32) {
            float hi[8], lo[8];
            if (g == 0) {
#pragma unroll
              for (int i = 0; i < 8; ++i) { hi[i] = s0[i]; lo[i] = s1[i]; }
            } else {
              tmem_ld8(hcol + c0, hi);
              tmem_ld8(lcol + c0, lo);
#pragma unroll
              for (int i = 0; i < 8; ++i) {       // two-sum of hi and the group's value
                const float sum = hi[i] + s0[i];
                const float bv = sum - hi[i];
                lo[i] += (hi[i] - (sum - bv)) + (s0[i] - bv) + s1[i];
                hi[i] = sum;
              }
            }
            if (g == G - 1) {
              double* C = reinterpret_cast<double*>(out.p);
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                const int64_t n = n0 + c0 + i;
                if (mok && n < N) {
                  const int64_t off = base + n * out.cs;
                  if ((uint64_t)off < (uint64_t)out.limit) {
                    const double v = (double)hi[i] + (double)lo[i];
                    double* o = C + off;
                    *o = out.accumulate ? *o + v : v;
                  } else {
                    oob = true;
                  }
                }
              }
            } else {
              tmem_st8(hcol + c0, hi);
              tmem_st8(lcol + c0, lo);
            }
          }
        }
        if constexpr (MODE != TG_STORE_F32) asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) bar_arrive(&acc_empty[gg & 1]);
      }
      if (oob) atomicExch(err, 2);
      if (!ok) break;
      if constexpr (MODE == TG_STORE_F32) {
        if (out.omax) {
          const unsigned int mb = __reduce_max_sync(0xffffffffu, __float_as_uint(vmax));
          if (lane == 0 && mb) atomicMax(reinterpret_cast<unsigned int*>(out.omax) + z, mb);
        }
      }
    }
  }
  if (!ok) {
    *abrt = 1;
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// tiled map over (k, row[, batch]) with a box of 16 x box_rows (x 1); zeros outside
ttg_status make_map(CUtensorMap* map, const TOperand& o, int box_rows, bool* three_d) {
  auto fn = encode_fn();
  if (!fn) return TTG_CUDA_ERR;
  if (!o.p || !o.amax || o.rows <= 0 || o.kext <= 0 || o.ld < o.kext || (o.ld * 4) % 16 != 0 ||
      (reinterpret_cast<uintptr_t>(o.p) & 15) != 0 || o.batch < 0 ||
      (o.batch > 0 && ((o.bstride * 4) % 16 != 0 || o.bstride <= 0)))
    return TTG_BAD_ARG;
  *three_d = o.batch > 0;
  cuuint64_t dims[3] = {(cuuint64_t)o.kext, (cuuint64_t)o.rows,
                        (cuuint64_t)(o.batch > 0 ? o.batch : 1)};
  cuuint64_t strides[2] = {(cuuint64_t)o.ld * 4, (cuuint64_t)o.bstride * 4};
  cuuint32_t box[3] = {(cuuint32_t)TG_K, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, *three_d ? 3 : 2,
                        const_cast<float*>(o.p), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? TTG_OK : TTG_BAD_ARG;
}

template <int MODE>
ttg_status launch_mode(int grid, cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb,
                       bool a3, bool b3, const TOperand& A, const TOperand& B, int Z, int G,
                       int kg, TileSched sch, const TOut& out, int* err) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_tgemm<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
  });
  if (attr != cudaSuccess) return TTG_CUDA_ERR;
  k_tgemm<MODE><<<grid, kThreads, kSmem, st>>>(ma, mb, a3 ? 1 : 0, b3 ? 1 : 0, A.amax, B.amax,
                                               (int)A.rows, (int)B.rows, Z, G, kg, sch, out, err);
  TTG_COUNT();
  cudaError_t e = cudaGetLastError();
  // TTG_SYNC_LAUNCHES=1: wait for each contraction and report its own error
  // (debugging: a fault is then charged to the launch that caused it)
  if (e == cudaSuccess && sync_launches()) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fprintf(stderr, "ttg: k_tgemm<%d> (grid %d, M %lld, N %lld, Z %d, G %d, kg %d) failed: %s\n",
            MODE, grid, (long long)A.rows, (long long)B.rows, Z, G, kg, cudaGetErrorString(e));
    return TTG_CUDA_ERR;
  }
  return TTG_OK;
}

// amax[g] = max |x[r][k]| over rows r < rows and k in [g gk, (g+1) gk) within kext
__global__ void k_group_max(const float* __restrict__ x, int64_t rows, int64_t kext, int64_t ld,
                            int64_t gk, float* __restrict__ amax) {
  const int g = blockIdx.y;
  const int64_t k0 = (int64_t)g * gk, k1 = min(kext, k0 + gk);
  float vmax = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < rows * (k1 - k0);
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / (k1 - k0), k = k0 + e % (k1 - k0);
    vmax = fmaxf(vmax, fabsf(x[r * ld + k]));
  }
  const unsigned int mb = __reduce_max_sync(0xffffffffu, __float_as_uint(vmax));
  if ((threadIdx.x & 31) == 0 && mb) atomicMax(reinterpret_cast<unsigned int*>(amax) + g, mb);
}

}  // namespace

ttg_status tgemm(cudaStream_t st, int mode, const TOperand& A, const TOperand& B, int Z, int G,
                 int kg, const TOut& out, int* err) {
  if (Z <= 0 || G <= 0 || kg <= 0 || kg * TG_K > 192 || !out.p || !err || out.r1 <= 0 ||
      out.limit <= 0)
    return TTG_BAD_ARG;
  if (mode == TG_STORE_F32 && G != 1) return TTG_BAD_ARG;
  if (mode == TG_SQSUM_F64 && (Z != 1 || A.batch < G || !out.w)) return TTG_BAD_ARG;
  if ((A.batch > 0 && A.batch < Z) || (B.batch > 0 && B.batch < Z)) return TTG_BAD_ARG;
  if (A.rows > INT32_MAX || B.rows > INT32_MAX) return TTG_BAD_ARG;
  CUtensorMap ma, mb;
  bool a3, b3;
  TTG_TRY(make_map(&ma, A, TG_M, &a3));
  TTG_TRY(make_map(&mb, B, TG_N, &b3));
  TileSched sch{(int)((A.rows + TG_M - 1) / TG_M), (int)((B.rows + TG_N - 1) / TG_N)};
  const int64_t ntiles = (int64_t)sch.tiles_m * sch.tiles_n * Z;
  int dev = 0, sms = 0;
  TTG_CUDA_TRY(cudaGetDevice(&dev));
  TTG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = (int)std::min<int64_t>(ntiles, sms);
  switch (mode) {
    case TG_STORE_F32:
      return launch_mode<TG_STORE_F32>(grid, st, ma, mb, a3, b3, A, B, Z, G, kg, sch, out, err);
    case TG_SUM_F64:
      return launch_mode<TG_SUM_F64>(grid, st, ma, mb, a3, b3, A, B, Z, G, kg, sch, out, err);
    case TG_SQSUM_F64:
      return launch_mode<TG_SQSUM_F64>(grid, st, ma, mb, a3, b3, A, B, Z, G, kg, sch, out, err);
  }
  return TTG_BAD_ARG;
}

}  // namespace ttg

extern "C" ttg_status ttg_tc_gemm(int64_t m, int64_t n, int64_t k, const float* a_dev,
                                  int64_t lda, const float* b_dev, int64_t ldb, int32_t groups,
                                  double* c_dev, int64_t ldc, void* stream) {
  using namespace ttg;
  if (m <= 0 || n <= 0 || k <= 0 || !a_dev || !b_dev || !c_dev || lda < k || ldb < k ||
      ldc < n || groups <= 0)
    return TTG_BAD_ARG;
  const int64_t gk = (k + groups - 1) / groups;              // K values per group
  const int kg = (int)((gk + TG_K - 1) / TG_K);              // chunks per group
  const int64_t gw = (int64_t)kg * TG_K;                     // groups are whole chunks
  if (groups > 1 && gw * (groups - 1) >= k) return TTG_BAD_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DevBuf am, err;
  TTG_TRY(am.alloc((size_t)2 * groups * 4));
  TTG_TRY(err.alloc(sizeof(int)));
  TTG_CUDA_TRY(cudaMemsetAsync(am.p, 0, (size_t)2 * groups * 4, st));
  TTG_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  k_group_max<<<dim3(64, groups), 256, 0, st>>>(a_dev, m, k, lda, gw, am.as<float>()); TTG_COUNT();
  k_group_max<<<dim3(64, groups), 256, 0, st>>>(b_dev, n, k, ldb, gw, am.as<float>() + groups); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  TOperand A{a_dev, m, k, lda, 0, 0, am.as<float>()};
  TOperand B{b_dev, n, k, ldb, 0, 0, am.as<float>() + groups};
  TOut o{c_dev, m + 1, ldc, 0, 1, 0};
  o.limit = (m - 1) * ldc + n;
  TTG_TRY(tgemm(st, TG_SUM_F64, A, B, 1, groups, kg, o, err.as<int>()));
  int e = 0;
  TTG_CUDA_TRY(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  return e == 0 ? TTG_OK : e == 2 ? TTG_BAD_ARG : e == 3 ? TTG_CUDA_ERR : TTG_TIMEOUT;
}
