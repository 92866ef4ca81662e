// Tensor-core contraction of FP32 operands (tgemm.cu), used by the Hartree
// kernel expansion and the density build.
#pragma once

#include <cstdint>

#include "ttg.h"

namespace ttg {

// One K-contiguous FP32 operand: `rows` rows of `kext` values, row stride
// `ld` elements (a multiple of 4), optionally `batch` matrices `bstride`
// elements apart (batch 0 = one matrix shared by every batch index).
// Values beyond kext or rows read as zero.  amax: max |value| of each slice
// the contraction cuts on a common grid -- per group for TG_SUM_F64 (and for
// A in TG_SQSUM_F64), else per batch (one entry when not batched); an
// over-estimate is allowed (it costs low-order bits), an under-estimate is not.
struct TOperand {
  const float* p = nullptr;
  int64_t rows = 0, kext = 0, ld = 0;
  int64_t batch = 0, bstride = 0;
  const float* amax = nullptr;
};

// Where C(m, n) of batch z goes: element offset
//   (m % r1) * s1 + (m / r1) * s2 + n * cs + z * bs.
struct TOut {
  void* p = nullptr;
  int64_t r1 = 1, s1 = 0, s2 = 0, cs = 0, bs = 0;
  const float* w = nullptr;   // TG_SQSUM_F64: weight of each group
  int accumulate = 0;         // FP64 outputs: add to C instead of overwriting it
  float* omax = nullptr;      // TG_STORE_F32: max |C| per batch (atomicMax into zeroed words)
  int64_t limit = 0;          // elements of C that may be written: a store at an offset
                              // outside [0, limit) is skipped and sets err to 2
};

enum TgemmMode {
  TG_STORE_F32 = 0,   // one group; C stored as FP32
  TG_SUM_F64 = 1,     // G groups summed in double-FP32; C stored as FP64
  TG_SQSUM_F64 = 2,   // sum over groups g of w[g] (group product)^2 in double-FP32,
                      // group g reading batch g of A (B shared); C stored as FP64
};

// C(m, n, z) = sum_{g < G} sum_{k in group g} A(m, k, z) B(n, k, z) with
// m < A.rows, n < B.rows, z < Z.  Group g covers K-chunks [g kg, (g+1) kg) of
// 16 values (TG_SQSUM_F64: every group covers chunks [0, kg) of A's batch g),
// at most 192 values per group.  `err` is a device int set to 1 when a
// bounded wait ran out, to 2 when a store fell outside out.limit, to 3 when
// a copy barrier was found out of phase (the kernel stops issuing work).
ttg_status tgemm(cudaStream_t st, int mode, const TOperand& A, const TOperand& B, int Z, int G,
                 int kg, const TOut& out, int* err);

}  // namespace ttg
