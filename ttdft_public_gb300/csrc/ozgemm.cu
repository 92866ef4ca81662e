// FP64-accurate GEMMs of the orthonormalisation and Rayleigh-Ritz steps on the
// tcgen05 tensor cores: the Gram matrices X^T X and X^T (H X), the update
// X L^-T and the rotation X Q (eigensolver/MultTm.cu:86-224, main.cc:1066-1207
// compute them in FP64).
//
// C[m][n] (+)= sum_k A(m, k) B(n, k) with FP64 operands A (M x K) and B
// (N x K), each stored K-major (element (r, k) at p[r ld + k]) or MN-major
// (p[k ld + r]); C is FP64 at C[m c_rs + n c_cs].
//
// Arithmetic (an Ozaki-type error-free split).  Every row r of an operand has
// a power-of-two scale with max_k |A(r, k)| < 2^e_r (k_rowexp_*, one pass
// over the operand).  The value v 2^(8 - e_r), below 256 in magnitude, is
// rounded to 40 fractional bits and written as six balanced base-256 digits
//   v 2^(8 - e_r) = d0 + d1 2^-8 + d2 2^-16 + ... + d5 2^-40,
//   |d0| <= 256, |d1..d5| <= 128,
// all exact in BF16.  The digits come from the double's bit pattern by
// integer operations: no FP64 arithmetic, which runs at a small fraction of
// the FP32 rate on this part.  The product of two values is sum_{i,j} d_i d'_j 2^-8(i+j);
// the 21 digit products with i + j <= 5 are summed per level L = i + j in six
// FP32 accumulators in tensor memory.  Over a group of 96 values of K a level
// sum is an integer of magnitude below 96 * 2^17 < 2^24, so the accumulators
// hold it exactly.  The epilogue folds the six levels of a group with
// error-free two-sums and adds the groups in double-FP32 (about 2^-48
// relative).  Left out: the digit products with i + j >= 6 and the rounding
// of each value to 2^-40 of its row's scale, each below 2^-47 of the product
// of the two rows' scales.
//
// One CTA per output tile of 128 x 32 and K range (split K), warp-specialised:
//  - warp 0, one thread: TMA tile loads of the FP64 operands (box 16 x 128 of
//    A, 16 x 32 of B, either layout) into a raw ring of 3 stages;
//  - warp 3, one thread: waits for the raw copies in order and publishes the
//    count of landed chunks (one thread polls the barriers, not eight warps);
//  - warps 4-11, each an eighth of the rows of every chunk: cut the 160 rows x
//    16 values into six digit planes each, in the canonical K-major MMA
//    layout, into a ring of 5 stages;
//  - warp 2, one thread: waits for the digit planes (and, before a group, for
//    the epilogue to have emptied the accumulator buffer it will use) and
//    publishes the count of ready chunks;
//  - warp 1, one thread: 21 MMAs (M128 N32 K16) per chunk into the six level
//    accumulators of one of two buffers;
//  - warps 12-15 (one per 32 TMEM lanes): fold the levels of each group into
//    running double-FP32 sums in registers; at the end scale by
//    2^(e_m + e_n - 16) and store.
// Every wait is bounded; a wait that runs out sets the error word and the
// abort flag, after which no role issues new copies or MMAs and the CTA
// drains what it issued before releasing tensor memory.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "ttg_internal.cuh"
#include "tc_common.cuh"

namespace ttg {
namespace {

using namespace tc;

constexpr int OZ_M = 128;                               // rows of an A tile (MMA M)
constexpr int OZ_N = 32;                                // rows of a B tile (MMA N)
constexpr int OZ_K = 16;                                // K per chunk
constexpr int kDigits = 6;
constexpr int kLevels = 6;
constexpr int kGroupChunks = 6;                         // 96 values of K per exact level sum
constexpr int kRawA = OZ_M * OZ_K * 8;                  // 16 KB FP64
constexpr int kRawB = OZ_N * OZ_K * 8;                  // 4 KB
constexpr int kRawStage = kRawA + kRawB;                // 20 KB
constexpr int kPlA = OZ_M * OZ_K * 2;                   // 4 KB: one BF16 digit plane of A
constexpr int kPlB = OZ_N * OZ_K * 2;                   // 1 KB
constexpr int kSplStage = kDigits * (kPlA + kPlB);      // 30 KB
constexpr int kRawStages = 3;
constexpr int kSplStages = 5;
constexpr int kSmem = kRawStages * kRawStage + kSplStages * kSplStage + 1024;
constexpr int kConvWarp0 = 4, kConvWarps = 8;           // share every chunk's rows
constexpr int kEpiWarp0 = 12, kEpiWarps = 4;
constexpr int kThreads = (kEpiWarp0 + kEpiWarps) * 32;  // 512
constexpr int kBufCols = kLevels * OZ_N;                // 192
constexpr uint32_t kTmemCols = 512;                     // two buffers (384)

// kind::f16: BF16 x BF16 -> FP32, A and B K-major, M = 128, N = 32
__device__ __forceinline__ uint32_t idesc_oz() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_N >> 3) << 17) |
         ((uint32_t)(OZ_M >> 4) << 24);
}

// Six balanced base-256 digits of v 2^(8 - e) (see the file comment) from the
// bits of v; zero for zeros and subnormals (below 2^-1022, far under the
// 2^-40 resolution of any row whose scale is a normal number); NaN in, NaN out.
// One 64-bit shift places the 48-bit fixed-point value; the digits come from
// its two 24-bit halves with 32-bit integer operations.
__device__ __forceinline__ void digits6(double v, int e, int adj, float* d) {
  const int hi = __double2hiint(v);
  const uint32_t lo = (uint32_t)__double2loint(v);
  int E = (hi >> 20) & 0x7FF;
  if (E == 0x7FF) {
#pragma unroll
    for (int i = 0; i < kDigits; ++i) d[i] = __int_as_float(0x7fc00000);
    return;
  }
  uint32_t xl = 0, xh = 0;
  if (E != 0) E = min(E + adj, 2046);                    // v 2^adj (a K scale)
  if (E > 0) {
    const unsigned long long M =
        ((unsigned long long)((hi & 0xFFFFF) | 0x100000) << 32) | lo;
    // v 2^(8-e) 2^40 = M 2^(E - 1075 + 48 - e); |v| < 2^e makes the shift >= 5
    const int rs = 1075 - 48 + e - E;
    if (rs < 63) {
      const unsigned long long X = (M + (1ull << (rs - 1))) >> rs;   // rounded, < 2^48 + 1
      xl = (uint32_t)X & 0xFFFFFFu;
      xh = (uint32_t)(X >> 24);
    }
  }
  // balanced digits, lowest first: d = ((t + 128) mod 256) - 128, t <- (t + 128) / 256
  int t = (int)xl, g[kDigits];
  g[5] = ((t + 128) & 255) - 128; t = (t + 128) >> 8;
  g[4] = ((t + 128) & 255) - 128; t = (t + 128) >> 8;
  g[3] = ((t + 128) & 255) - 128; t = (t + 128) >> 8;
  int u = (int)xh + t;
  g[2] = ((u + 128) & 255) - 128; u = (u + 128) >> 8;
  g[1] = ((u + 128) & 255) - 128; u = (u + 128) >> 8;
  g[0] = u;                                             // 0 .. 256
  const int sm = hi >> 31;                              // 0 or -1
#pragma unroll
  for (int i = 0; i < kDigits; ++i) d[i] = (float)((g[i] ^ sm) - sm);
}

// three 8-column tensor-memory loads and one wait, in one statement (the
// registers are defined only after the wait)
__device__ __forceinline__ void tmem_ld8x3(uint32_t a0, uint32_t a1, uint32_t a2, float* v0,
                                           float* v1, float* v2) {
  uint32_t r[24];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%24];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%25];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%26];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23])
      : "r"(a0), "r"(a1), "r"(a2)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    v0[j] = __uint_as_float(r[j]);
    v1[j] = __uint_as_float(r[8 + j]);
    v2[j] = __uint_as_float(r[16 + j]);
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);   // integers <= 256: exact
  return *reinterpret_cast<const uint32_t*>(&h);
}

// byte offset of element (row, k) in a canonical K-major digit plane
__device__ __forceinline__ int plane_off(int row, int k) {
  return (row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// Digit planes of one block of 8 operand rows of a chunk (raw FP64 tile of
// R rows, either layout) by one warp.  Lane (r8, kp) = (lane / 4, lane % 4)
// takes the pairs (row 8 rb + r8, k = 8 kh + 2 kp, k + 1), kh = 0, 1: the 32
// lanes of a step store to 32 different banks of each plane (plane_off).
template <int R, int MN>
__device__ __forceinline__ void slice_block(const double* __restrict__ raw, const int* es,
                                            unsigned char* planes, int plane_bytes, int rb,
                                            int lane, const int* __restrict__ kadj, int ksign) {
  const int row = 8 * rb + (lane >> 2), kp = lane & 3;
  const int e = es[row];
  double v[2][2];
#pragma unroll
  for (int kh = 0; kh < 2; ++kh) {
    const int k = 8 * kh + 2 * kp;
    if (MN) {                 // raw [k][row]
      v[kh][0] = raw[k * R + row];
      v[kh][1] = raw[(k + 1) * R + row];
    } else {                  // raw [row][16]
      const double2 vv = *reinterpret_cast<const double2*>(raw + row * OZ_K + k);
      v[kh][0] = vv.x;
      v[kh][1] = vv.y;
    }
  }
#pragma unroll
  for (int kh = 0; kh < 2; ++kh) {
    const int k = 8 * kh + 2 * kp;
    float d0[kDigits], d1[kDigits];
    const int a0 = kadj ? ksign * __ldg(kadj + k) : 0;
    const int a1 = kadj ? ksign * __ldg(kadj + k + 1) : 0;
    digits6(v[kh][0], e, a0, d0);
    digits6(v[kh][1], e, a1, d1);
    const int off = plane_off(row, k);
#pragma unroll
    for (int d = 0; d < kDigits; ++d)
      *reinterpret_cast<uint32_t*>(planes + d * plane_bytes + off) = pack_bf16(d0[d], d1[d]);
  }
}

struct OzTiles {
  int tiles_m, tiles_n;
  int sym;          // only tiles with n0 <= m0 + 127 (on and below the diagonal)
  __device__ void at(int t, int& mt, int& nt) const {
    if (!sym) {
      mt = t / tiles_n;
      nt = t - mt * tiles_n;
      return;
    }
    int m = 0;
    for (;; ++m) {
      const int row = min(4 * m + 4, tiles_n);
      if (t < row) break;
      t -= row;
    }
    mt = m;
    nt = t;
  }
};

template <int A_MN, int B_MN>
__global__ void __launch_bounds__(kThreads, 1) k_ozgemm(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
    const int* __restrict__ expA, const int* __restrict__ expB, int M, int N, int K,
    int k_per_split, int b_lower, OzTiles tiles, double* __restrict__ out, int64_t o_rs,
    int64_t o_cs, int64_t o_zs, const int* __restrict__ kexp, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (su32(smem_raw) & 1023)) & 1023);
  unsigned char* raw = smem;                                  // kRawStages x 20 KB
  unsigned char* spl = smem + kRawStages * kRawStage;         // kSplStages x 30 KB
  __shared__ __align__(8) uint64_t raw_full[kRawStages], raw_empty[kRawStages];
  __shared__ __align__(8) uint64_t spl_full[kSplStages], spl_empty[kSplStages];
  __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2];
  __shared__ __align__(8) uint64_t fin;
  __shared__ uint32_t tmem_slot;
  __shared__ uint32_t ready, landed;
  __shared__ int abort_flag;
  __shared__ int eA[OZ_M], eB[OZ_N];                          // row scales 2^e
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int mt, nt;
  tiles.at(blockIdx.x, mt, nt);
  const int m0 = mt * OZ_M, n0 = nt * OZ_N;
  const int k0 = blockIdx.y * k_per_split;
  int k1 = min(K, k0 + k_per_split);
  if (b_lower) k1 = min(k1, n0 + OZ_N);                       // B(n, k) = 0 for k > n
  const int nq = k1 > k0 ? (k1 - k0 + OZ_K - 1) / OZ_K : 0;  // chunks
  const int ng = (nq + kGroupChunks - 1) / kGroupChunks;      // groups

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(su32(&tmem_slot)), "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 32) {
    for (int s = 0; s < kRawStages; ++s) {
      bar_init(&raw_full[s], 1);
      bar_init(&raw_empty[s], kConvWarps);
    }
    for (int s = 0; s < kSplStages; ++s) {
      bar_init(&spl_full[s], kConvWarps);
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
  for (int i = tid; i < OZ_M; i += blockDim.x) {
    eA[i] = m0 + i < M ? __ldg(expA + m0 + i) : 0;
  }
  for (int i = tid; i < OZ_N; i += blockDim.x) {
    eB[i] = n0 + i < N ? __ldg(expB + n0 + i) : 0;
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
      int q = 0;
      for (; q < nq; ++q) {
        const int s = q % kRawStages;
        if (q >= kRawStages &&
            !bar_wait(&raw_empty[s], (uint32_t)((q / kRawStages - 1) & 1), abrt, 32)) {
          ok = false;
          break;
        }
        // the stage's previous copy must have landed before it is armed again
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
        const int kc = k0 + q * OZ_K;
        if (A_MN) tma_load(dst, &tmA, m0, kc, 0, false, fb);
        else tma_load(dst, &tmA, kc, m0, 0, false, fb);
        if (B_MN) tma_load(dst + kRawA, &tmB, n0, kc, 0, false, fb);
        else tma_load(dst + kRawA, &tmB, kc, n0, 0, false, fb);
      }
      if (!ok)
        for (int r = (q > kRawStages ? q - kRawStages : 0); r < q; ++r)
          bar_drain(&raw_full[r % kRawStages], (uint32_t)((r / kRawStages) & 1));
    }
  } else if (warp == 3) {
    // ---- raw copies landed, in order
    if (lane == 0) {
      for (int q = 0; q < nq; ++q) {
        if (!bar_wait(&raw_full[q % kRawStages], (uint32_t)((q / kRawStages) & 1), abrt, 32)) {
          ok = false;
          break;
        }
        asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(su32(&landed)),
                     "r"((uint32_t)(q + 1)) : "memory");
      }
    }
  } else if (warp >= kConvWarp0 && warp < kConvWarp0 + kConvWarps) {
    // ---- digit planes: every converter warp takes its share of the rows of
    // every chunk (row blocks of 8: cw, cw + 8, ...), so a chunk's raw stage
    // is released after an eighth of the work; each warp waits on every phase
    // of the barriers it uses, in order
    const int cw = warp - kConvWarp0;
    for (int q = 0; q < nq; ++q) {
      const int s = q % kRawStages, s2 = q % kSplStages;
      bool w = true;
      if (lane == 0) {
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
        if (w && q >= kSplStages)
          w = bar_wait(&spl_empty[s2], (uint32_t)((q / kSplStages - 1) & 1), abrt, 32);
      }
      w = __shfl_sync(0xffffffffu, w, 0);
      if (!w) { ok = false; break; }
      const double* ra = reinterpret_cast<const double*>(raw + s * kRawStage);
      const double* rb = reinterpret_cast<const double*>(raw + s * kRawStage + kRawA);
      unsigned char* dst = spl + s2 * kSplStage;
      for (int blk = cw; blk < (OZ_M + OZ_N) / 8; blk += kConvWarps) {
        // K scales of this chunk (K values beyond the operands are zero)
        const int* kq = kexp ? kexp + (k0 + q * OZ_K) : nullptr;
        if (blk < OZ_M / 8) slice_block<OZ_M, A_MN>(ra, eA, dst, kPlA, blk, lane, kq, -1);
        else slice_block<OZ_N, B_MN>(rb, eB, dst + kDigits * kPlA, kPlB, blk - OZ_M / 8, lane, kq,
                                     1);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        bar_arrive(&raw_empty[s]);
        bar_arrive(&spl_full[s2]);
      }
    }
  } else if (warp == 2) {
    // ---- digit planes ready (and accumulator buffers emptied), in order
    if (lane == 0) {
      for (int q = 0; q < nq && ok; ++q) {
        const int g = q / kGroupChunks;
        if (q % kGroupChunks == 0 && g >= 2 &&
            !bar_wait(&acc_empty[g & 1], (uint32_t)(((g >> 1) - 1) & 1), abrt, 32)) {
          ok = false;
          break;
        }
        if (!bar_wait(&spl_full[q % kSplStages], (uint32_t)((q / kSplStages) & 1), abrt, 16)) {
          ok = false;
          break;
        }
        asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(su32(&ready)),
                     "r"((uint32_t)(q + 1)) : "memory");
      }
    }
  } else if (warp == 1) {
    // ---- MMA issue: 21 digit products per chunk into six level accumulators
    if (lane == 0) {
      const uint32_t idesc = idesc_oz();
      const uint32_t spl0 = su32(spl);
      uint32_t avail = 0;
      for (int q = 0; q < nq; ++q) {
        const int g = q / kGroupChunks, c = q % kGroupChunks;
        const uint32_t dbuf = tmem + (uint32_t)((g & 1) * kBufCols);
        for (int i = 0; i < kTcMaxWait && avail <= (uint32_t)q; ++i) {
          asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(avail)
                       : "r"(su32(&ready)) : "memory");
          if (avail > (uint32_t)q || *abrt) break;
          __nanosleep(16);
        }
        if (avail <= (uint32_t)q) { ok = false; *abrt = 1; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t base = spl0 + (uint32_t)((q % kSplStages) * kSplStage);
        int p = 0;
#pragma unroll
        for (int L = kLevels - 1; L >= 0; --L) {
#pragma unroll
          for (int i = 0; i <= L; ++i, ++p) {
            const int j = L - i;
            const uint64_t da = kmajor_desc(base + i * kPlA);
            const uint64_t db = kmajor_desc(base + kDigits * kPlA + j * kPlB);
            const uint32_t acc = (c > 0 || i > 0) ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                ::"r"(dbuf + (uint32_t)(L * OZ_N)), "l"(da), "l"(db), "r"(idesc), "r"(acc));
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
            ::"r"(su32(&spl_empty[q % kSplStages])) : "memory");
        if (c == kGroupChunks - 1 || q == nq - 1)
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
              ::"r"(su32(&acc_full[g & 1])) : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(su32(&fin)) : "memory");
      bar_drain(&fin, 0);
    }
  } else if (warp >= kEpiWarp0) {
    // ---- epilogue: TMEM lanes 32 (warp & 3) .., all 32 columns
    const int qd = warp & 3;
    const int row = qd * 32 + lane;
    const uint32_t lanes = (uint32_t)(qd * 32) << 16;
    float hi[OZ_N], lo[OZ_N];
#pragma unroll
    for (int c = 0; c < OZ_N; ++c) { hi[c] = 0.f; lo[c] = 0.f; }
    for (int g = 0; g < ng; ++g) {
      if (!bar_wait(&acc_full[g & 1], (uint32_t)((g >> 1) & 1), abrt, 64)) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acol = tmem + lanes + (uint32_t)((g & 1) * kBufCols);
#pragma unroll
      for (int c0 = 0; c0 < OZ_N; c0 += 8) {
        float S[kLevels][8];
        tmem_ld8x3(acol + c0, acol + OZ_N + c0, acol + 2 * OZ_N + c0, S[0], S[1], S[2]);
        tmem_ld8x3(acol + 3 * OZ_N + c0, acol + 4 * OZ_N + c0, acol + 5 * OZ_N + c0, S[3], S[4],
                   S[5]);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          // S0 + S1 2^-8 + ... + S5 2^-40 as (h, l), then into (hi, lo)
          float h = S[0][i], l = 0.f;
          float sc = 1.f / 256.f;
#pragma unroll
          for (int L = 1; L < kLevels; ++L, sc *= (1.f / 256.f)) {
            const float t = S[L][i] * sc;
            const float h2 = h + t;
            const float bv = h2 - h;
            l += (h - (h2 - bv)) + (t - bv);
            h = h2;
          }
          const float sum = hi[c0 + i] + h;
          const float bv = sum - hi[c0 + i];
          lo[c0 + i] += (hi[c0 + i] - (sum - bv)) + (h - bv) + l;
          hi[c0 + i] = sum;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) bar_arrive(&acc_empty[g & 1]);
    }
    if (ok && m0 + row < M) {
      const int em = eA[row];
#pragma unroll
      for (int c = 0; c < OZ_N; ++c) {
        const int n = n0 + c;
        if (n < N) {
          const double v = ((double)hi[c] + (double)lo[c]) * ldexp(1.0, em + eB[c] - 16);
          out[(int64_t)blockIdx.y * o_zs + (int64_t)(m0 + row) * o_rs + (int64_t)n * o_cs] = v;
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

// Row scales: e[r] with max_k |A(r, k)| < 2^e[r] (0 for an all-zero row), from
// the largest biased exponent of the row: any v with biased exponent E is
// below 2^(E - 1022).  ebits[r] (zeroed by the caller) collects the maxima.
// With K scales (kexp, ksign): the biased exponent of v 2^(ksign kexp[k]).
__device__ __forceinline__ int scaled_ebits(double v, const int* kexp, int ksign, int64_t k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  int E = (int)((b >> 52) & 0x7FF);
  if (E != 0 && E != 0x7FF && kexp) E = max(0, min(2046, E + ksign * __ldg(kexp + k)));
  return E;
}

__global__ void k_rowexp_mn(const double* __restrict__ p, int64_t rows, int64_t kext, int64_t ld,
                            int64_t k_per_block, const int* __restrict__ kexp, int ksign,
                            int* __restrict__ ebits) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int64_t k0 = (int64_t)blockIdx.y * k_per_block;
  const int64_t k1 = min(kext, k0 + k_per_block);
  int m = 0;
  for (int64_t k = k0; k < k1; ++k) m = max(m, scaled_ebits(p[k * ld + r], kexp, ksign, k));
  if (m) atomicMax(ebits + r, m);
}

// K-major rows: one warp per row
__global__ void k_rowexp_k(const double* __restrict__ p, int64_t rows, int64_t kext, int64_t ld,
                           const int* __restrict__ kexp, int ksign, int* __restrict__ ebits) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  int m = 0;
  for (int64_t k = lane; k < kext; k += 32) m = max(m, scaled_ebits(p[r * ld + k], kexp, ksign, k));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) ebits[r] = m;
}

__global__ void k_exp_from_bits(int* __restrict__ e, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int b = e[i];
    // a NaN or Inf row (b = 2047) keeps a large scale: its digits are NaN anyway
    e[i] = b == 0 ? 0 : min(b, 2046) - 1022;
  }
}

// S = sum of the split partials (column-major M x N); sym: tiles above the
// diagonal were not computed, S[m, n] is read from [n, m] there.
__global__ void k_oz_reduce(const double* __restrict__ part, int nsplit, int M, int N, int sym,
                            double* __restrict__ C, int64_t c_rs, int64_t c_cs) {
  const int64_t mn = (int64_t)M * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < mn;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(i % M), n = (int)(i / M);
    int64_t src = i;
    if (sym && (n / OZ_N) * OZ_N > (m / OZ_M) * OZ_M + OZ_M - 1) src = n + (int64_t)m * M;
    double s = 0.0;
    for (int z = 0; z < nsplit; ++z) s += part[(int64_t)z * mn + src];
    C[m * c_rs + n * c_cs] = s;
  }
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

bool map_ok(const OzOperand& o) {
  return o.p && o.rows > 0 && o.kext > 0 && (o.ld * 8) % 16 == 0 &&
         (reinterpret_cast<uintptr_t>(o.p) & 15) == 0 &&
         (o.mn_major ? o.ld >= o.rows : o.ld >= o.kext);
}

ttg_status make_map(CUtensorMap* map, const OzOperand& o, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return TTG_CUDA_ERR;
  cuuint64_t dims[2], strides[1] = {(cuuint64_t)o.ld * 8};
  cuuint32_t box[2], es[2] = {1, 1};
  if (o.mn_major) {
    dims[0] = (cuuint64_t)o.rows;
    dims[1] = (cuuint64_t)o.kext;
    box[0] = (cuuint32_t)box_rows;
    box[1] = (cuuint32_t)OZ_K;
  } else {
    dims[0] = (cuuint64_t)o.kext;
    dims[1] = (cuuint64_t)o.rows;
    box[0] = (cuuint32_t)OZ_K;
    box[1] = (cuuint32_t)box_rows;
  }
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(o.p), dims,
                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? TTG_OK : TTG_BAD_ARG;
}

ttg_status row_exps(cudaStream_t st, const OzOperand& o, int* e, const int* kexp = nullptr,
                    int ksign = 0) {
  TTG_CUDA_TRY(cudaMemsetAsync(e, 0, (size_t)o.rows * sizeof(int), st));
  if (o.mn_major) {
    const int64_t kb = 256;                 // enough CTAs for a narrow block of many rows
    dim3 grid((unsigned)((o.rows + 255) / 256), (unsigned)((o.kext + kb - 1) / kb));
    k_rowexp_mn<<<grid, 256, 0, st>>>(o.p, o.rows, o.kext, o.ld, kb, kexp, ksign, e); TTG_COUNT();
  } else {
    k_rowexp_k<<<(unsigned)((o.rows * 32 + 255) / 256), 256, 0, st>>>(o.p, o.rows, o.kext, o.ld,
                                                                     kexp, ksign, e); TTG_COUNT();
  }
  TTG_CUDA_TRY(cudaGetLastError());
  k_exp_from_bits<<<(unsigned)((o.rows + 255) / 256), 256, 0, st>>>(e, o.rows); TTG_COUNT();
  TTG_CUDA_TRY(cudaGetLastError());
  return TTG_OK;
}

template <int A_MN, int B_MN>
ttg_status launch(dim3 grid, cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb,
                  const int* ea, const int* eb, int M, int N, int K, int kps, int b_lower,
                  OzTiles tiles, double* out, int64_t o_rs, int64_t o_cs, int64_t o_zs,
                  const int* kexp, int* err) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_ozgemm<A_MN, B_MN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmem);
  });
  if (attr != cudaSuccess) return TTG_CUDA_ERR;
  k_ozgemm<A_MN, B_MN><<<grid, kThreads, kSmem, st>>>(ma, mb, ea, eb, M, N, K, kps, b_lower,
                                                     tiles, out, o_rs, o_cs, o_zs, kexp, err);
  TTG_COUNT();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && sync_launches()) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fprintf(stderr, "ttg: k_ozgemm<%d, %d> (M %d, N %d, K %d) failed: %s\n", A_MN, B_MN, M, N, K,
            cudaGetErrorString(e));
    return TTG_CUDA_ERR;
  }
  return TTG_OK;
}

}  // namespace

bool ozgemm_supported(const OzOperand& A, const OzOperand& B) {
  if (getenv("TTG_DISABLE_OZGEMM")) return false;
  return map_ok(A) && map_ok(B) && A.kext == B.kext && A.rows <= INT32_MAX &&
         B.rows <= INT32_MAX && A.kext <= INT32_MAX;
}

ttg_status ozgemm(ttg_op* op, const OzOperand& A, const OzOperand& B, double* C, int64_t c_rs,
                  int64_t c_cs, bool sym, bool b_lower, const OzOperand* kscale_of) {
  if (!ozgemm_supported(A, B) || !C) return TTG_BAD_ARG;
  if (sym && A.rows != B.rows) return TTG_BAD_ARG;
  cudaStream_t st = op->stream;
  const int M = (int)A.rows, N = (int)B.rows, K = (int)A.kext;
  if (op->oz_exp.bytes < (size_t)(M + N) * sizeof(int))
    TTG_TRY(op->oz_exp.alloc((size_t)(M + N) * sizeof(int)));
  if (!op->oz_err.p) {
    TTG_TRY(op->oz_err.alloc(sizeof(int)));
    TTG_CUDA_TRY(cudaMemsetAsync(op->oz_err.p, 0, sizeof(int), st));
  }
  int* ea = op->oz_exp.as<int>();
  int* eb = ea + M;
  // K scales: the row scales of kscale_of (an MN-major view whose rows are
  // the K index), A scaled by 2^-f_k and B by 2^f_k; the buffer is padded
  // with zeros to whole chunks
  const int* kexp = nullptr;
  if (kscale_of) {
    if (kscale_of->rows != K) return TTG_BAD_ARG;
    const size_t kb = (size_t)((K + OZ_K - 1) / OZ_K * OZ_K) * sizeof(int);
    if (op->oz_kexp.bytes < kb) TTG_TRY(op->oz_kexp.alloc(kb));
    TTG_CUDA_TRY(cudaMemsetAsync(op->oz_kexp.p, 0, kb, st));
    TTG_TRY(row_exps(st, *kscale_of, op->oz_kexp.as<int>()));
    kexp = op->oz_kexp.as<int>();
  }
  TTG_TRY(row_exps(st, A, ea, kexp, -1));
  if (!kexp && B.p == A.p && B.rows == A.rows && B.kext == A.kext && B.ld == A.ld &&
      B.mn_major == A.mn_major)
    TTG_CUDA_TRY(cudaMemcpyAsync(eb, ea, (size_t)M * sizeof(int), cudaMemcpyDeviceToDevice, st));
  else
    TTG_TRY(row_exps(st, B, eb, kexp, 1));
  CUtensorMap ma, mb;
  TTG_TRY(make_map(&ma, A, OZ_M));
  TTG_TRY(make_map(&mb, B, OZ_N));
  OzTiles tiles{(M + OZ_M - 1) / OZ_M, (N + OZ_N - 1) / OZ_N, sym ? 1 : 0};
  int64_t ntiles = (int64_t)tiles.tiles_m * tiles.tiles_n;
  if (sym) {
    ntiles = 0;
    for (int m = 0; m < tiles.tiles_m; ++m) ntiles += std::min(4 * m + 4, tiles.tiles_n);
  }
  // split K so that the CTAs (one per SM) fill the GPU a few times over
  const int groupk = kGroupChunks * OZ_K;
  const int64_t kgroups = (K + groupk - 1) / groupk;
  int nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(kgroups, (4 * 152 + ntiles - 1) / ntiles));
  if (b_lower) nsplit = 1;
  const int kps = (int)(((kgroups + nsplit - 1) / nsplit) * groupk);
  nsplit = (int)((K + kps - 1) / kps);
  double* out = C;
  int64_t o_rs = c_rs, o_cs = c_cs;
  if (nsplit > 1 || sym) {
    const size_t need = (size_t)nsplit * M * N * sizeof(double);
    if (op->partial.bytes < need) TTG_TRY(op->partial.alloc(need));
    out = op->partial.as<double>();
    o_rs = 1;
    o_cs = M;
  }
  if (ntiles > INT32_MAX || nsplit > 65535) return TTG_BAD_ARG;
  const dim3 grid((unsigned)ntiles, (unsigned)nsplit);
  const int64_t zs = (out == C) ? 0 : (int64_t)M * N;
  int* err = op->oz_err.as<int>();
  const int bl = b_lower ? 1 : 0;
  if (A.mn_major && B.mn_major)
    TTG_TRY((launch<1, 1>(grid, st, ma, mb, ea, eb, M, N, K, kps, bl, tiles, out, o_rs, o_cs, zs, kexp, err)));
  else if (A.mn_major)
    TTG_TRY((launch<1, 0>(grid, st, ma, mb, ea, eb, M, N, K, kps, bl, tiles, out, o_rs, o_cs, zs, kexp, err)));
  else if (B.mn_major)
    TTG_TRY((launch<0, 1>(grid, st, ma, mb, ea, eb, M, N, K, kps, bl, tiles, out, o_rs, o_cs, zs, kexp, err)));
  else
    TTG_TRY((launch<0, 0>(grid, st, ma, mb, ea, eb, M, N, K, kps, bl, tiles, out, o_rs, o_cs, zs, kexp, err)));
  if (out != C) {
    const int64_t mn = (int64_t)M * N;
    k_oz_reduce<<<(unsigned)std::min<int64_t>((mn + 255) / 256, 4096), 256, 0, st>>>(
        out, nsplit, M, N, sym ? 1 : 0, C, c_rs, c_cs); TTG_COUNT();
    TTG_CUDA_TRY(cudaGetLastError());
  }
  return TTG_OK;
}

ttg_status ozgemm_error(ttg_op* op) {
  if (!op->oz_err.p) return TTG_OK;
  int e = 0;
  TTG_CUDA_TRY(cudaMemcpyAsync(&e, op->oz_err.p, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  if (e) {
    TTG_CUDA_TRY(cudaMemsetAsync(op->oz_err.p, 0, sizeof(int), op->stream));
    fprintf(stderr, "ttg: FP64 tensor-core GEMM: %s\n",
            e == 3 ? "a copy barrier out of phase" : "a bounded wait ran out");
    return e == 3 ? TTG_CUDA_ERR : TTG_TIMEOUT;
  }
  return TTG_OK;
}

}  // namespace ttg
