// Chebyshev filter degrees on the fifth-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory): Ynew = alpha (H Y) + beta Y +
// delta X (ChebyShevFilter.cc:97-170).  FP32 degrees run FP32-accurate on
// BF16 MMAs (three-term split below); BF16 degrees run one BF16 product.
//
// Tiles.  128 rows per tile (a 4 x 4 x 8 block of the Tucker index, or 128
// consecutive rows without Tucker ranks); the tile's sorted column union is
// padded to chunks of 16 slots.  A chunk is one MMA step: M = 128 rows,
// N = k states, K = 16 slots.
//
// Precision (FP32 degrees).  Every FP32 value v is split into three BF16 terms
// v = v0 + v1 + v2 (exact for normal values; |v1| <= 2^-8 |v|,
// |v2| <= 2^-17 |v|).  The product H Y is accumulated in FP32 from the six
// term products of order <= 2 (v0w0, v0w1, v1w0, v1w1, v0w2, v2w0); the three
// dropped ones are below 2^-24 of |v w| together, so the result carries FP32
// accuracy at BF16 MMA rates.
//
// Data movement per chunk.
//  - H: the three BF16 planes of the chunk (128 x 16 values each, already in
//    the canonical K-major no-swizzle layout of the MMA operand) are one
//    contiguous 12 KB block, copied by one bulk asynchronous copy (TMA,
//    L2 evict-first) into the H ring.
//  - Y: the 16 source rows are gathered from three BF16 planes of the block
//    (written by k_split3 before the launch) with 16-byte cp.async copies
//    (L2 evict-last: rows are re-read by many tiles) into the row ring, in
//    the MN-major operand layout with the 128-byte swizzle: 8 lanes read one
//    whole 128-byte piece of a row, so one instruction moves four rows.
// Warp roles (10 warps, one CTA per SM):
//  - warp 0, one thread: the H copies, up to nh (8-12) chunks ahead;
//  - warps 3-9: the row gathers, whole chunks in turn; a warp waits for its
//    own copies and fences them for the async proxy before it arrives;
//  - warp 2, one thread: waits for each chunk's "full" mbarrier in order and
//    publishes the count of ready chunks in shared memory;
//  - warp 1, one thread: six MMAs (one for BF16) and one commit (to the chunk's "done"
//    mbarrier) per chunk.  It never waits on an mbarrier itself: such a wait
//    queues behind its outstanding MMAs (about 0.1 us per chunk).
// Waits off the critical path back off with nanosleep: tight polling by many
// threads slows every mbarrier operation of the CTA.  After the last chunk,
// warps 0-3 (one per 32 TMEM lanes) read the accumulator from tensor memory
// and apply the recurrence in FP32.
// BF16 degrees (NT = 1) use H's plane 0 (its BF16 rounding), gather the
// BF16 block's rows as they are, issue one MMA per chunk and round the
// epilogue's FP32 result to BF16.
// Every wait (mbarrier or the ready count) is bounded; a wait that runs out
// sets an error word.

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>
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
constexpr int kMaxH = 12;                     // H ring stages (12 KB each)
constexpr int kMaxB = 8;                      // gathered-row ring stages
constexpr int kSmemBudget = 227 * 1024 - 1024;
constexpr int kThreads = 320;                // 10 warps
constexpr int kHWarp = 0;                     // lane 0 copies the H blocks
constexpr int kMmaWarp = 1;                   // lane 0 issues the MMAs
constexpr int kWaitWarp = 2;                  // waits for full stages on the MMA warp's behalf
constexpr int kFirstBWarp = 3;                // warps 3-9 gather the block's rows
constexpr int kBWarps = 7;
constexpr int kMaxWait = 1 << 20;
constexpr int kColAhead = 4;                  // chunks per warp whose column indices are loaded ahead
constexpr int kAtom = 64;                     // states per 128-byte swizzle row
constexpr int kAtomBytes = 16 * 128;          // one atom of a chunk: 16 slot rows x 128 bytes

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

// B operand (slots x states, states contiguous) in the 128-byte swizzle
// layout: per 64-state atom 16 slot rows of 128 bytes, the 16-byte piece j of
// row s stored at piece j ^ (s % 8); rows 8-15 1024 bytes after rows 0-7
// (stride byte offset), atoms 2048 bytes apart (leading byte offset).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)(kAtomBytes >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;                 // 128-byte swizzle
  return d;
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

// For waits off the critical path: a thread that polls an mbarrier without
// pause slows the mbarrier operations of the threads that are on it.
__device__ __forceinline__ bool mbar_wait_idle(uint64_t* b, uint32_t parity, int ns) {
  for (int i = 0; i < kMaxWait; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    if (ok) return true;
    __nanosleep(ns);
  }
  return false;
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// NT = 3: FP32 degree (three BF16 terms of H and of the block, six
// products); NT = 1: BF16 degree (H rounded to BF16, the BF16 block itself,
// one product).  TIO is the block's element type (float / bf16).
template <int NT, typename TIO>
__global__ void __launch_bounds__(kThreads) k_cheb_umma(
    const int64_t* __restrict__ tptr, const int* __restrict__ tcol, const int* __restrict__ rowmap,
    const int* __restrict__ order, const __nv_bfloat16* __restrict__ hpl,
    const __nv_bfloat16* __restrict__ xpl, int64_t pstride, int ps, const TIO* __restrict__ src,
    const TIO* xold, TIO* dst, int k, int64_t ld, float alpha, float beta, float delta,
    uint32_t tmem_cols, int nh, int nb, int* __restrict__ err) {
  constexpr int HB = NT * 2 * PLANE_ELEMS;    // H bytes per chunk: the first NT planes
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // rings start on a 1024-byte boundary (swizzle atoms; descriptor base offset 0):
  // nb gathered-row stages, then nh H stages
  unsigned char* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  // full[c % nd]: both stages of chunk c have landed (the H copy by bytes and
  // an arrive each from the H and row producers); done[c % nd]: the MMAs of
  // chunk c have read them.  nd >= nh, nb: a producer refilling for chunk c
  // has waited for chunk c - nh or c - nb, so chunk c - nd's phase is over.
  __shared__ __align__(8) uint64_t full[kMaxH], done[kMaxH];
  __shared__ __align__(8) uint64_t accf;     // all MMAs of the tile done (one phase)
  __shared__ uint32_t tmem_slot;
  __shared__ uint32_t ready;                 // chunks whose two stages are full
  // tiles in decreasing chunk count, so the longest start first and the short
  // ones fill the tail of the launch
  const int tile = __ldg(order + blockIdx.x), tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int natoms = (k + kAtom - 1) / kAtom;
  const int bplane = natoms * kAtomBytes;               // one gathered plane
  const int bstage = NT * bplane;
  unsigned char* hring = smem + nb * bstage;
  const int64_t c_first = tptr[tile] / UK;
  const int nch = (int)((tptr[tile + 1] - tptr[tile]) / UK);
  const int ngrp = k >> 3;
  const int nd = max(nh, nb);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_slot)), "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < nd; ++s) {
      mbar_init(&full[s], 2);                    // H expect_tx arrive + the rows' warp
      mbar_init(&done[s], 1);                    // one tcgen05.commit
    }
    mbar_init(&accf, 1);
    ready = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  bool ok = true;

  if (warp == kHWarp) {
    // H ring: one thread copies chunk c's H block into stage c % nh once the
    // MMAs of chunk c - nh have read it, running up to nh chunks ahead of the
    // MMAs (the H copies come from HBM and are the slowest to land)
    if (lane == 0) {
      uint64_t pol_stream;
      asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol_stream));
      for (int c = 0; c < nch; ++c) {
        const int s = c % nh;
        // one wait per two chunks: the MMAs complete in order, so chunk
        // c + 1 - nh done means chunk c - nh is done too
        if (c >= nh && ((c - nh) & 1) == 0) {
          const int x = (c + 1 < nch ? c + 1 : c) - nh;
          ok &= mbar_wait(&done[x % nd], (x / nd) & 1);
        }
        const uint32_t fb = smem_u32(&full[c % nd]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb),
                     "r"(HB) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
            " [%0], [%1], %2, [%3], %4;"
            ::"r"(smem_u32(hring + s * HB)), "l"(hpl + (c_first + c) * CHUNK_ELEMS),
              "r"(HB), "r"(fb), "l"(pol_stream)
            : "memory");
      }
    }
  } else if (warp >= kFirstBWarp) {
    // gathered rows: warps kFirstBWarp.. (pw = 0 .. np-1) take whole chunks in
    // turn, chunk c to warp c % np, into stage c % nb once the MMAs of chunk
    // c - nb have read it.  np <= nb keeps every wait within one phase of the
    // stage's "free" barrier (a warp's previous chunk c - np waited for chunk
    // c - np - nb >= c - 2 nb).  A warp waits for its own copies, fences them
    // for the tensor core's (async-proxy) reads and arrives on the stage's
    // "full" barrier; the np warps fill np stages at once.
    const int np = min(kBWarps, nb);
    const int pw = warp - kFirstBWarp;
    if (pw < np) {
      // lane = row of a quad (lane / 8) x 16-byte piece of a 128-byte row
      // (lane % 8): one instruction reads four whole 128-byte rows and writes
      // four 128-byte rows of shared memory (128-byte swizzle: piece j of
      // slot row s lands at piece j ^ (s % 8))
      const int lr = lane >> 3, lj = lane & 7;
      uint64_t pol_keep;     // the block's rows are re-read by many tiles
      asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_keep));
      const int* colp = tcol + c_first * UK + (lane & 15);
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
          const int s = c % nb;
          if (c >= nb) ok &= mbar_wait_idle(&done[(c - nb) % nd], ((c - nb) / nd) & 1, 64);
          const uint32_t sb = smem_u32(smem + s * bstage);
#pragma unroll
          for (int rq = 0; rq < 4; ++rq) {
            const int srow = 4 * rq + lr;                    // slot of this lane's row
            const int64_t col = __shfl_sync(0xffffffffu, cur[j], srow);
            const __nv_bfloat16* xs = xpl + col * ps + 8 * lj;
            const uint32_t drow = sb + (uint32_t)((srow >> 3) * 1024 + (srow & 7) * 128 +
                                                  ((lj ^ (srow & 7)) << 4));
            for (int a = 0; a < natoms; ++a) {
              if (a * 8 + lj < ngrp) {
#pragma unroll
                for (int pl = 0; pl < NT; ++pl)
                  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;"
                               ::"r"(drow + (uint32_t)(pl * bplane + a * kAtomBytes)),
                                 "l"(xs + pl * pstride + a * kAtom), "l"(pol_keep)
                               : "memory");
              }
            }
          }
          cp_async_commit();
          cp_async_wait<0>();
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&full[c % nd]))
                         : "memory");
        }
#pragma unroll
        for (int j = 0; j < kColAhead; ++j) cur[j] = nxt[j];
      }
      cp_async_wait<0>();
    }
  } else if (warp == kWaitWarp) {
    // waits for each chunk's stages to fill, in order, and publishes the count of
    // ready chunks to the MMA thread: an mbarrier wait by the MMA-issuing
    // thread itself queues behind its outstanding MMAs (about 0.1 us a chunk)
    if (lane == 0) {
      for (int c = 0; c < nch; ++c) {
        ok &= mbar_wait(&full[c % nd], (c / nd) & 1);
        asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(smem_u32(&ready)), "r"(c + 1)
                     : "memory");
      }
    }
  } else if (warp == kMmaWarp && lane == 0) {
    // MMA thread: six MMAs per chunk (term pairs, smallest products first),
    // committed to the chunk's "done" barrier.  Its per-chunk work is kept to
    // a short dependency chain (stage addresses and descriptors advance by
    // additions): the issue of the next chunk waits on it.
    const uint32_t idesc = instr_desc(UR, k);
    const uint64_t da_hi = smem_desc(0), db_hi = smem_desc_sw128(0);
    const uint32_t a_first = smem_u32(hring) >> 4, b_first = smem_u32(smem) >> 4;
    const uint32_t a_end = a_first + nh * (HB >> 4);
    const uint32_t b_end = b_first + nb * (bstage >> 4);
    const uint32_t bpl = (uint32_t)bplane >> 4, apl = (2 * PLANE_ELEMS) >> 4;
    const uint32_t done0 = smem_u32(&done[0]);
    uint32_t a_lo = a_first, b_lo = b_first;
    int sd = 0;
    uint32_t avail = 0;
    for (int c = 0; c < nch; ++c) {
      for (int i = 0; i < kMaxWait && avail <= (uint32_t)c; ++i)
        asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(avail) : "r"(smem_u32(&ready))
                     : "memory");
      ok &= avail > (uint32_t)c;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // (term of A, term of B): (1,1) (0,2) (2,0) (0,1) (1,0) (0,0)
      const uint64_t da[6] = {da_hi | (a_lo + apl), da_hi | a_lo, da_hi | (a_lo + 2 * apl),
                              da_hi | a_lo, da_hi | (a_lo + apl), da_hi | a_lo};
      const uint64_t db[6] = {db_hi | (b_lo + bpl), db_hi | (b_lo + 2 * bpl), db_hi | b_lo,
                              db_hi | (b_lo + bpl), db_hi | b_lo, db_hi | b_lo};
      constexpr int q0 = NT == 3 ? 0 : 5;       // NT = 1: (0,0) only
#pragma unroll
      for (int q = q0; q < 6; ++q) {
        const uint32_t acc = (c > 0 || q > q0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
            ::"r"(tmem), "l"(da[q]), "l"(db[q]), "r"(idesc), "r"(acc));
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(done0 + 8 * sd)
          : "memory");
      a_lo += HB >> 4;
      if (a_lo == a_end) a_lo = a_first;
      b_lo += bstage >> 4;
      if (b_lo == b_end) b_lo = b_first;
      if (++sd == nd) sd = 0;
    }
    if (nch > 0)
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          ::"r"(smem_u32(&accf))
          : "memory");
  }
  __syncwarp();
  // all MMAs done.  A barrier of its own, used for one phase: a thread may
  // get here long before the last chunk's stage barriers have passed the
  // phase before their last one, where a parity wait on them would pass early.
  if (nch > 0) ok &= mbar_wait_idle(&accf, 0, 512);
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
      if constexpr (std::is_same<TIO, float>::value) {
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
      } else {
        // BF16 block: 8 values (16 bytes) per access, arithmetic in FP32
#pragma unroll
        for (int j = 0; j < 16; j += 8) {
          const uint4 yu = *reinterpret_cast<const uint4*>(src + off + j);
          uint4 xu = make_uint4(0u, 0u, 0u, 0u);
          if (delta != 0.f) xu = *reinterpret_cast<const uint4*>(xold + off + j);
          const __nv_bfloat162* y2 = reinterpret_cast<const __nv_bfloat162*>(&yu);
          const __nv_bfloat162* x2 = reinterpret_cast<const __nv_bfloat162*>(&xu);
          uint4 ou;
          __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&ou);
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const float2 yf = __bfloat1622float2(y2[t]);
            const float2 xf = __bfloat1622float2(x2[t]);
            const float a0 = fmaf(delta, xf.x, alpha * __uint_as_float(v[j + 2 * t]) + beta * yf.x);
            const float a1 = fmaf(delta, xf.y, alpha * __uint_as_float(v[j + 2 * t + 1]) + beta * yf.y);
            o2[t] = __floats2bfloat162_rn(a0, a1);
          }
          *reinterpret_cast<uint4*>(dst + off + j) = ou;
        }
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
  // Launch order.  While the gathered rows of one launch (three BF16 planes
  // of up to 256 states per row) fit in L2, tiles run longest first, so the
  // short ones fill the tail.  Beyond that they run in their spatial order
  // (x fastest, then y, then z): the ~152 tiles resident at a time then
  // cover one slab of the Tucker grid, and the rows their columns gather
  // (the slab plus the band of H around it) stay in L2 while the slab is
  // worked on, instead of being fetched from HBM for every tile.
  std::vector<int32_t> order(ntiles);
  for (int64_t t = 0; t < ntiles; ++t) order[t] = (int32_t)t;
  const int64_t gather_bytes = n * (int64_t)std::min(op->max_k, 256) * 6;
  if (gather_bytes <= ((int64_t)64 << 20))
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return tptr[a + 1] > tptr[b + 1]; });
  for (int64_t t = 0; t < ntiles; ++t) tptr[t + 1] += tptr[t];
  const int64_t slots = tptr[ntiles];
  const int64_t nchunk = slots / UK;
  const bool keep = op->keep_pattern;
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
            if (keep && pass == 0) pos[hp[r] + e] = (int32_t)slot;   // slot within the tile
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
    // row -> tile * 128 + lane of the row in its tile
    std::vector<int32_t> urow(n, -1);
    for (int64_t t = 0; t < ntiles; ++t)
      for (int m = 0; m < UR; ++m)
        if (rowmap[t * UR + m] >= 0) urow[rowmap[t * UR + m]] = (int32_t)(t * UR + m);
    TTG_TRY(op->pattern.umma_row.alloc(n * sizeof(int32_t)));
    TTG_CUDA_TRY(cudaMemcpyAsync(op->pattern.umma_row.p, urow.data(), n * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, op->stream));
    op->device_bytes += op->pattern.umma_pos.bytes + op->pattern.umma_row.bytes;
  }
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  op->device_bytes += U.tptr.bytes + U.tcol.bytes + U.rowmap.bytes + U.order.bytes + U.hpl.bytes;
  return TTG_OK;
}

bool umma_supported(const ttg_op* op, int prec, int k) {
  return (prec == TTG_PREC_FP32 || prec == TTG_PREC_BF16) && op->umma.n_tiles > 0 && !op->tc_disabled && k >= 16 &&
         k <= 256 && k % 16 == 0 && k <= op->ld;
}

namespace {

template <int NT, typename TIO>
ttg_status launch_umma_t(ttg_op* op, const __nv_bfloat16* xpl, int64_t pstride, int ps,
                         const void* src, const void* xold, void* dst, int k, double alpha,
                         double beta, double delta) {
  UmmaOp& U = op->umma;
  constexpr int HB = NT * 2 * PLANE_ELEMS;
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_cheb_umma<NT, TIO>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBudget);
  });
  if (attr_err != cudaSuccess) return TTG_CUDA_ERR;
  uint32_t cols = 32;
  while ((int)cols < k) cols <<= 1;
  const int natoms = (k + kAtom - 1) / kAtom;
  const int bstage = NT * natoms * kAtomBytes;
  // eight H stages (the H copies run ahead of the rows), the rest to the
  // row stages, then what is left to more H stages (1024 bytes go to alignment)
  const int avail = kSmemBudget - 1024;
  const int nb = std::min(kMaxB, (avail - 8 * HB) / bstage);
  const int nh = std::min(kMaxH, (avail - nb * bstage) / HB);
  if (nb < 3 || nh < 3) return TTG_BAD_ARG;
  const size_t smem = (size_t)nb * bstage + (size_t)nh * HB + 1024;
  TTG_TRY(kt_begin(op, NT == 3 ? TTG_KT_UMMA_FP32 : TTG_KT_UMMA_BF16));
  k_cheb_umma<NT, TIO><<<(unsigned)U.n_tiles, kThreads, smem, op->stream>>>(
      U.tptr.as<int64_t>(), U.tcol.as<int>(), U.rowmap.as<int>(), U.order.as<int>(),
      U.hpl.as<__nv_bfloat16>(), xpl, pstride, ps, reinterpret_cast<const TIO*>(src),
      reinterpret_cast<const TIO*>(xold), reinterpret_cast<TIO*>(dst), k, op->ld, (float)alpha,
      (float)beta, (float)delta, cols, nh, nb, U.err.as<int>()); TTG_COUNT();
  TTG_LAUNCHED(op);
  TTG_TRY(kt_end(op));
  return TTG_OK;
}

}  // namespace

ttg_status launch_cheb_umma(ttg_op* op, int prec, const void* src, const void* xold, void* dst,
                            int k, double alpha, double beta, double delta) {
  UmmaOp& U = op->umma;
  const int64_t rows = op->n + op->nproj;
  if (prec == TTG_PREC_BF16)   // the block's rows are gathered as they are (row stride ld)
    return launch_umma_t<1, __nv_bfloat16>(op, reinterpret_cast<const __nv_bfloat16*>(src), 0,
                                           (int)op->ld, src, xold, dst, k, alpha, beta, delta);
  const int ps = k;                                  // multiple of 16
  const int64_t pstride = rows * ps;
  const size_t need = (size_t)3 * pstride * sizeof(uint16_t);
  if (U.xpl.bytes < need) {
    TTG_TRY(U.xpl.alloc(need));
    op->device_bytes += (int64_t)need;
  }
  const int grid_s = (int)std::min<int64_t>((rows * ps + 255) / 256, 152 * 16);
  k_split3<<<grid_s, 256, 0, op->stream>>>(reinterpret_cast<const float*>(src), rows, k, op->ld,
                                           U.xpl.as<__nv_bfloat16>(), ps, pstride); TTG_COUNT();
  TTG_LAUNCHED(op);
  return launch_umma_t<3, float>(op, U.xpl.as<__nv_bfloat16>(), pstride, ps, src, xold, dst, k,
                                 alpha, beta, delta);
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
