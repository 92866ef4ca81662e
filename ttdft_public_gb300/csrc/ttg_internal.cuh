// Internal declarations shared by the libttg translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <atomic>

#include "ttg.h"

#define TTG_CUDA_TRY(call)                                                  \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      fprintf(stderr, "ttg: %s failed: %s (%s:%d)\n", #call,                \
              cudaGetErrorString(e_), __FILE__, __LINE__);                  \
      return e_ == cudaErrorMemoryAllocation ? TTG_OOM : TTG_CUDA_ERR;      \
    }                                                                       \
  } while (0)

#define TTG_TRY(call)                 \
  do {                                \
    ttg_status s_ = (call);           \
    if (s_ != TTG_OK) return s_;      \
  } while (0)

// Every kernel launch of the library bumps one process-wide counter
// (ttg_kernel_launches); TTG_LAUNCHED also counts per operator.
#define TTG_COUNT() (::ttg::g_kernel_launches.fetch_add(1, std::memory_order_relaxed))

// Checks the last launch; counts it.  With TTG_SYNC_LAUNCHES set in the
// environment it also waits for the kernel, so that a fault is reported at
// the launch that caused it (debugging only: it serialises the host).
#define TTG_LAUNCHED(op)                                                    \
  do {                                                                      \
    (op)->launches++;                                                       \
    cudaError_t e_ = cudaGetLastError();                                    \
    if (e_ == cudaSuccess && ::ttg::sync_launches())                        \
      e_ = cudaDeviceSynchronize();                                         \
    if (e_ != cudaSuccess) {                                                \
      fprintf(stderr, "ttg: launch failed: %s (%s:%d)\n",                   \
              cudaGetErrorString(e_), __FILE__, __LINE__);                  \
      return TTG_CUDA_ERR;                                                  \
    }                                                                       \
  } while (0)

namespace ttg {
extern std::atomic<long long> g_kernel_launches;

inline bool sync_launches() {
  static const bool on = getenv("TTG_SYNC_LAUNCHES") != nullptr;
  return on;
}

constexpr int kGroupRows = 8;       // rows per row group of the SpMM format
constexpr int kMaxSlots = 16;
constexpr int kMaxLanczos = 512;    // Lanczos steps (T is at most this size)
// op->scal layout, in doubles
constexpr int64_t kScalLanczos = 0;      // alpha/beta pairs, 2*kMaxLanczos
constexpr int64_t kScalFermi = 1024;     // mu, iterations, residual
constexpr int64_t kScalEig = 2048;       // eigenvalues (k)
constexpr int64_t kScalJacobi = 2048 + 4096;  // unsorted eigenvalues (k)

// Device buffer owned by the library.
// Owning device allocation: freed by release() or when it goes out of scope.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  ttg_status alloc(size_t n);
  void release();
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Row-group sliced format of H_ext = [H_loc | C^T] (N x (N + nproj)).
// Group g holds rows [g*G, g*G+G).  Its merged column list is the sorted
// union of the rows' column indices, padded to a multiple of 4 slots; slot s
// stores one column index and G values (one per row, 0 where absent), so
// that one load of a source row feeds G rows.  Columns >= N address the
// projector rows W = D*C*Y that are stored right after the block's N rows.
struct RowGroups {
  int64_t n_groups = 0;
  int64_t slots = 0;
  DevBuf gptr;     // int64 [n_groups+1], slot offsets
  DevBuf gcol;     // int32 [slots]
  DevBuf v64;      // double [slots*G]
  DevBuf v32;      // float  [slots*G]
  DevBuf v16;      // bf16   [slots*G]
  DevBuf vdf;      // float2 [slots*G]: FP64 values as (hi, lo) FP32 pairs
};

// 3-D row tiles of 64 rows for the tensor-core SpMM (spmm_tc.cu): per tile a
// merged column list in chunks of 16 slots, H values pre-arranged in MMA
// B-fragment order (FP32 for TF32, BF16), and the tile's original row ids.
struct TileOp {
  int64_t n_tiles = 0;
  int64_t slots = 0;
  DevBuf tptr;     // int64 [n_tiles+1], slot offsets (multiples of 16)
  DevBuf tcol;     // int32 [slots]
  DevBuf rowmap;   // int32 [n_tiles*64], -1 = padding
  DevBuf v32;      // float, [chunk][8 n-tiles][32 lanes][4]
  DevBuf v16;      // bf16,  [chunk][8 n-tiles][32 lanes][4]
};

// 128-row tiles for the tcgen05 filter degrees (spmm_umma.cu): H as three
// BF16 planes per 16-slot chunk in the MMA operand layout (FP32 degrees use
// all three, BF16 degrees plane 0), and the block's three BF16 planes that
// the FP32 degrees gather.
struct UmmaOp {
  int64_t n_tiles = 0;
  int64_t slots = 0;
  DevBuf tptr;     // int64 [n_tiles+1], slot offsets (multiples of 16)
  DevBuf tcol;     // int32 [slots]
  DevBuf rowmap;   // int32 [n_tiles*128], -1 = padding
  DevBuf order;    // int32 [n_tiles], launch order: most chunks first
  DevBuf hpl;      // bf16 [chunk][3][128 x 16]
  DevBuf xpl;      // bf16 [3][n + nproj][k]
  DevBuf err;      // int: a bounded wait of the kernel ran out
};

// The fixed sparsity pattern of H_loc and where each entry lives in the device
// formats, kept when the operator is created with Tucker ranks so that its
// values can be recomputed on the device for a new potential (hupdate.cu).
struct Pattern {
  DevBuf row_ptr;    // int64 [n+1]
  DevBuf col;        // int32 [nnz]
  DevBuf rg_pos;     // int32 [nnz]: slot of the entry within its row group's column list
  DevBuf tile_base;  // int32 [nnz]: lane base of the entry's tile fragment
  DevBuf tile_slot;  // uint8 [nnz]: slot of the entry within its 16-slot chunk
  DevBuf umma_pos;   // int32 [nnz]: slot of the entry within its 128-row tile's column list
  DevBuf umma_row;   // int32 [n]: tile * 128 + lane of each row in the 128-row tiles
  int32_t r[3] = {0, 0, 0};   // Tucker ranks of the basis
  int32_t bw[3] = {0, 0, 0};  // max |coordinate difference| per direction over the entries
  DevBuf kin;        // 6 r x r 1-D matrices: DX DY DZ MX MY MZ (row-major)
  bool kinetic_set = false;
  DevBuf work;       // pair tables and the Tucker intermediates
  DevBuf work2;
};

// Device time of the fused filter-degree kernels, by kind (TTG_KT_*): with
// timing on, each such launch is bracketed by two events on the operator's
// stream; pairs are read back in batches, so timing never waits on the host.
struct KernelTimer {
  static constexpr int kPairs = 1024;
  bool on = false;
  std::vector<cudaEvent_t> ev;   // 2 * kPairs
  std::vector<int> kind;         // kind of each pending pair
  int used = 0;
  double ms[TTG_KT_KINDS] = {};
  long long count[TTG_KT_KINDS] = {};
};

// Work buffers of the Hartree kernel expansion (tensor.cu), grow-only and
// owned by the operator, so the SCF's calls allocate nothing once warm.
struct HartreeWork {
  DevBuf F[3];     // FP32 expansion factors (x, y: [t][i][a]; z: [l][t, c] with the weight)
  DevBuf gf;       // FP32 core, rows (b, c), a contiguous
  DevBuf p2;       // FP32 [t][(i, c)][b]
  DevBuf q;        // FP32 [(i, j)][(t, c)]
  int64_t q_layout[3] = {0, 0, 0};   // (rows, K, padded rank) the zeroed Q was laid out for
  DevBuf amax;     // FP32 group maxima of the operands (the tensor-core slicing grid)
  DevBuf err;      // int: a bounded wait of the tensor-core kernel ran out
};

// Work buffers of the density build (tensor.cu), grow-only, owned by the op.
struct DensityWork {
  DevBuf uf[3];    // FP32 basis values at the nodes, [i][a] (row stride a multiple of 4)
  DevBuf xt;       // FP32 block chunk, [s][(b, c)][a]
  DevBuf p1;       // FP32 [s][c][i][b]
  DevBuf p2;       // FP32 [s][j][i][c]
  DevBuf w;        // FP32 weights 2 f_s
  DevBuf amax;     // FP32 group maxima of the operands (the tensor-core slicing grid)
};

struct Csr {
  int64_t rows = 0, cols = 0, nnz = 0, max_row_nnz = 0;
  DevBuf ptr;      // int64
  DevBuf col;      // int32
  DevBuf val;      // double
  DevBuf val32;    // float
};

}  // namespace ttg

struct ttg_op {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t n = 0;
  int32_t nproj = 0;
  int32_t max_k = 0;
  int64_t nnz_h = 0, nnz_c = 0;
  ttg::RowGroups rg;
  ttg::TileOp tiles;          // tensor-core format (FP32/BF16 degrees)
  ttg::UmmaOp umma;           // tcgen05 format (FP32 and BF16 degrees)
  bool tc_disabled = false;   // TTG_DISABLE_TC=1: CUDA-core kernels only
  bool keep_pattern = false;  // Tucker ranks given: keep the pattern for value updates
  ttg::Pattern pattern;
  ttg::Csr C;                 // C (nproj x n) with D folded in: C_nloc = diag(D) C
  // workspace (rows = n + nproj, row-major, ld = max_k padded)
  int64_t ld = 0;             // row stride in elements of the working blocks
  ttg::DevBuf w32a, w32b;     // FP32 working blocks
  ttg::DevBuf w16a, w16b;     // BF16 working blocks
  ttg::DevBuf w64;            // FP64 scratch block (n + nproj rows)
  ttg::DevBuf wdf;            // float2 (hi, lo) copy of an FP64 block for the df64 SpMM
  ttg::DevBuf wpart;          // projector partial sums (nproj x splits x k)
  int rr_prec = TTG_PREC_DF64;  // arithmetic of the Rayleigh-Ritz product H X
  ttg::DevBuf kk0, kk1, kk2;  // k x k FP64 matrices
  ttg::DevBuf kk3;            // eigensolver scratch (k*k + 6k doubles)
  ttg::DevBuf chol;           // blocked Cholesky: the diagonal before factorisation
  ttg::DevBuf oz_exp;         // FP64 tensor-core GEMM: row scales of its operands
  ttg::DevBuf oz_kexp;        // FP64 tensor-core GEMM: K scales (padded to whole chunks)
  ttg::DevBuf oz_err;         // FP64 tensor-core GEMM: error word
  ttg::DevBuf eigbuf;         // eigensolver refinement (5 k*k doubles)
  ttg::DevBuf eigf;           // FP32 tridiagonalisation scratch
  ttg::DevBuf partial;        // split-K partials for the Gram
  ttg::DevBuf sth_a, sth_b, sth_part, sth_part2;  // STHOSVD work (grow-only)
  ttg::DevBuf scal;           // small FP64 scratch (reductions, status)
  ttg::DevBuf status;         // int32 device status words
  cudaEvent_t ev[ttg::kMaxSlots] = {};
  ttg::KernelTimer kt;
  ttg::HartreeWork hw;        // Hartree work buffers (ttg_hartree_device) and the
                              // tensor-core error word shared with the density
  ttg::DensityWork dw;        // density work buffers (ttg_density_device)
  int64_t launches = 0;
  int64_t shifted_orth = 0;   // shifted Cholesky-QR steps of ttg_chfsi_pass
  int64_t device_bytes = 0;
};

struct ttg_block {
  ttg_op* op = nullptr;
  int32_t k = 0;
  ttg::DevBuf x;              // FP64, (n + nproj) x ld row-major
};

namespace ttg {

// capi.cu: kernel timer (no-ops while timing is off)
ttg_status kt_begin(ttg_op* op, int kind);
ttg_status kt_end(ttg_op* op);

// spmm.cu
ttg_status build_row_groups(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                            const double* hv, int32_t nproj, const int64_t* cp,
                            const int32_t* cc, const double* cv, const double* d);
ttg_status launch_cheb_step(ttg_op* op, int prec, const void* src, const void* xold,
                            void* dst, int k, double alpha, double beta, double delta);
ttg_status launch_proj_w(ttg_op* op, int prec, void* src, int k);
ttg_status launch_apply_df64(ttg_op* op, const double* src, double* dst, int k);

// spmm_tc.cu
ttg_status build_tiles(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                       const double* hv, int32_t nproj, const int64_t* cp, const int32_t* cc,
                       const double* cv, const int32_t* dims);
bool tc_supported(const ttg_op* op, int prec, int k);
// spmm_umma.cu
ttg_status build_umma_tiles(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                            const double* hv, int32_t nproj, const int64_t* cp, const int32_t* cc,
                            const double* cv, const int32_t* dims);
bool umma_supported(const ttg_op* op, int prec, int k);
ttg_status launch_cheb_umma(ttg_op* op, int prec, const void* src, const void* xold, void* dst,
                            int k, double alpha, double beta, double delta);
ttg_status umma_check_error(ttg_op* op);
ttg_status launch_cheb_tc(ttg_op* op, int prec, const void* src, const void* xold, void* dst,
                          int k, double alpha, double beta, double delta);
ttg_status launch_convert(ttg_op* op, int from, int to, const void* src, void* dst,
                          int64_t rows, int k);

// tensor.cu: TTG_TIMEOUT (and clears the word) when a tensor-core launch of
// ttg_hartree_device or ttg_density_device gave up a bounded wait
ttg_status hartree_error(ttg_op* op);

// scf.cu: FP64 strided-batched GEMM (split-K when the output is small)
#ifdef __CUDACC__
// Double-FP32 ("df64") arithmetic: a value is an unevaluated sum hi + lo of
// two floats (about 48 significant bits).  FP64 runs at ~1.25 TFLOP/s on
// this part and FP32 at ~80, so the FP64 GEMMs run on the FP32 pipe in df64:
// one df64 multiply-add is 11 FP32 instructions (Dekker/Knuth error-free
// product and sum), about 5x the FP64 rate.  The product's lo x lo term
// (2^-48 relative) is dropped.
struct F2 {
  float h, l;
};

__device__ __forceinline__ F2 to_f2(double x) {
  const float h = (float)x;
  return F2{h, (float)(x - (double)h)};
}

// Folds lo into hi (fast two-sum; |lo| is at most a few ulps of hi).  The
// GEMM loops call it once per 16 steps of f2_fma: lo otherwise grows with
// the number of steps, and its own FP32 rounding then dominates the error
// of long sums (tests/test_df64_algorithm.py measures both).
__device__ __forceinline__ void f2_renorm(F2& acc) {
  const float s = acc.h + acc.l;
  acc.l = acc.l - (s - acc.h);
  acc.h = s;
}

// acc += a * b.  The accumulator is left unnormalised between renormalisations
// (lo is not folded into hi after every step): the loop-carried dependency is
// then a single FP32 add on hi and one on lo, and the sum is read out as
// (double)hi + (double)lo.  A 4096-term dot product lands within ~6e-14 of
// the sum of |terms| (FP32: ~4e-8), in a NumPy restatement of these steps.
__device__ __forceinline__ void f2_fma(F2& acc, F2 a, F2 b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);          // exact: a.h b.h = p + e
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = acc.h + p;             // two-sum of the high parts
  const float v = s - acc.h;
  const float t = (acc.h - (s - v)) + (p - v);
  acc.h = s;
  acc.l += t + e;
}

#endif

struct DOp {
  const double* p;
  int64_t rs, cs, bs;   // element strides: row (m or k), column (k or n), batch
};
ttg_status dgemm(cudaStream_t st, int M, int N, int K, int batch, DOp A, DOp B, double* C,
                 int64_t c_rs, int64_t c_cs, int64_t c_bs, DevBuf& scratch, bool sym = false);

// ozgemm.cu: FP64-accurate C = A B^T on the tensor cores (see the file).
// A FP64 operand: `rows` rows of `kext` values, K-major (element (r, k) at
// p[r ld + k]) or MN-major (p[k ld + r]); ld * 8 a multiple of 16.
struct OzOperand {
  const double* p;
  int64_t rows, kext, ld;
  bool mn_major;
};
// Whether ozgemm takes these operands (TMA alignment, sizes; off with
// TTG_DISABLE_OZGEMM); callers fall back to the double-FP32 CUDA-core GEMMs.
bool ozgemm_supported(const OzOperand& A, const OzOperand& B);
// C[m c_rs + n c_cs] = sum_k A(m, k) B(n, k).  sym: A B^T is symmetric (A = B,
// or B = H A): only tiles on and below the diagonal are computed and the
// others mirrored.  b_lower: B(n, k) = 0 for k > n (the sum stops at n).
// kscale_of: an MN-major operand whose rows are the K index (K of them);
// with power-of-two scales f_k = its row scales, A is sliced as
// A(m, k) 2^-f_k and B as B(n, k) 2^f_k, which leaves A B^T unchanged and
// keeps small K columns of A (that B amplifies) at full precision.
ttg_status ozgemm(ttg_op* op, const OzOperand& A, const OzOperand& B, double* C, int64_t c_rs,
                  int64_t c_cs, bool sym, bool b_lower = false,
                  const OzOperand* kscale_of = nullptr);
// Reads and clears the tensor-core GEMM's error word (synchronises).
ttg_status ozgemm_error(ttg_op* op);

// dense.cu
// S = X^T Y (k x k, column-major).  sym: S is known to be symmetric (X^T X,
// or X^T H X with H symmetric): only the tiles on and below the diagonal are
// computed and the others mirrored.
ttg_status gram_tn(ttg_op* op, const double* X, const double* Y, int k, double* S,
                   bool sym = false);
// out = X Q (transQ = 0) or X Q^T (transQ = 1); lower: Q is lower triangular
// (with transQ the sum over p stops at the output column)
ttg_status gemm_nn_small(ttg_op* op, const double* X, const double* Q, double* out, int k,
                         int transQ, bool lower = false);
ttg_status cholesky_inv(ttg_op* op, double* S, double* Linv, int k, int* d_status);
// S <- D^-1 S D^-1 + shift I with d = sqrt(diag S) written to d (k doubles);
// *bad (device int) counts diagonal entries that are not positive and finite
ttg_status unit_scale_shift(ttg_op* op, double* S, double* d, int k, double shift, int* bad);
// L[:, j] <- L[:, j] / d[j]
ttg_status scale_cols(ttg_op* op, double* L, const double* d, int k);
ttg_status syev_device(ttg_op* op, double* A, double* V, double* w, int k, int* d_status);
ttg_status sym_topk(ttg_op* op, double* A, int n, int r, double* w, double* U, int* d_status);
ttg_status colmajor_to_rows(ttg_op* op, const double* src, int64_t ld_src, double* dst,
                            int64_t ld_dst, int64_t n, int k);
ttg_status rows_to_colmajor(ttg_op* op, const double* src, int64_t ld_src, double* dst,
                            int64_t ld_dst, int64_t n, int k);
ttg_status lanczos_step(ttg_op* op, double* v, double* v0, const double* hv, double* ab, int it);
ttg_status normalize(ttg_op* op, double* v);
ttg_status fermi(ttg_op* op, const double* eig, int k, double ne, double kT, int max_iter,
                 double* occ, double* out);

}  // namespace ttg
