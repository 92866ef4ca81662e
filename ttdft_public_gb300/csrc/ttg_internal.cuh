// Internal declarations shared by the libttg translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <vector>

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

// Checks the last launch; counts it.
#define TTG_LAUNCHED(op)                                                    \
  do {                                                                      \
    (op)->launches++;                                                       \
    cudaError_t e_ = cudaGetLastError();                                    \
    if (e_ != cudaSuccess) {                                                \
      fprintf(stderr, "ttg: launch failed: %s (%s:%d)\n",                   \
              cudaGetErrorString(e_), __FILE__, __LINE__);                  \
      return TTG_CUDA_ERR;                                                  \
    }                                                                       \
  } while (0)

namespace ttg {

constexpr int kGroupRows = 8;       // rows per row group of the SpMM format
constexpr int kMaxSlots = 16;
constexpr int kMaxLanczos = 512;    // Lanczos steps (T is at most this size)
// op->scal layout, in doubles
constexpr int64_t kScalLanczos = 0;      // alpha/beta pairs, 2*kMaxLanczos
constexpr int64_t kScalFermi = 1024;     // mu, iterations, residual
constexpr int64_t kScalEig = 2048;       // eigenvalues (k)
constexpr int64_t kScalJacobi = 2048 + 4096;  // Jacobi rotation scratch

// Device buffer owned by the library.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
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
};

struct Csr {
  int64_t rows = 0, cols = 0, nnz = 0;
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
  ttg::Csr C;                 // C (nproj x n) with D folded in: C_nloc = diag(D) C
  // workspace (rows = n + nproj, row-major, ld = max_k padded)
  int64_t ld = 0;             // row stride in elements of the working blocks
  ttg::DevBuf w32a, w32b;     // FP32 working blocks
  ttg::DevBuf w16a, w16b;     // BF16 working blocks
  ttg::DevBuf w64;            // FP64 scratch block (n + nproj rows)
  ttg::DevBuf kk0, kk1, kk2;  // k x k FP64 matrices
  ttg::DevBuf partial;        // split-K partials for the Gram
  ttg::DevBuf scal;           // small FP64 scratch (reductions, status)
  ttg::DevBuf status;         // int32 device status words
  cudaEvent_t ev[ttg::kMaxSlots] = {};
  int64_t launches = 0;
  int64_t device_bytes = 0;
};

struct ttg_block {
  ttg_op* op = nullptr;
  int32_t k = 0;
  ttg::DevBuf x;              // FP64, (n + nproj) x ld row-major
};

namespace ttg {

// spmm.cu
ttg_status build_row_groups(ttg_op* op, int64_t n, const int64_t* hp, const int32_t* hc,
                            const double* hv, int32_t nproj, const int64_t* cp,
                            const int32_t* cc, const double* cv, const double* d);
ttg_status launch_cheb_step(ttg_op* op, int prec, const void* src, const void* xold,
                            void* dst, int k, double alpha, double beta, double delta);
ttg_status launch_proj_w(ttg_op* op, int prec, void* src, int k);
ttg_status launch_convert(ttg_op* op, int from, int to, const void* src, void* dst,
                          int64_t rows, int k);

// dense.cu
ttg_status gram_tn(ttg_op* op, const double* X, const double* Y, int k, double* S);
ttg_status gemm_nn_small(ttg_op* op, const double* X, const double* Q, double* out, int k,
                         int transQ);
ttg_status cholesky_inv(ttg_op* op, double* S, double* Linv, int k, int* d_status);
ttg_status syev_jacobi(ttg_op* op, double* A, double* V, double* w, int k, int* d_status);
ttg_status colmajor_to_rows(ttg_op* op, const double* src, int64_t ld_src, double* dst,
                            int64_t ld_dst, int64_t n, int k);
ttg_status rows_to_colmajor(ttg_op* op, const double* src, int64_t ld_src, double* dst,
                            int64_t ld_dst, int64_t n, int k);
ttg_status lanczos_step(ttg_op* op, double* v, double* v0, const double* hv, double* ab, int it);
ttg_status normalize(ttg_op* op, double* v);
ttg_status fermi(ttg_op* op, const double* eig, int k, double ne, double kT, int max_iter,
                 double* occ, double* out);

}  // namespace ttg
