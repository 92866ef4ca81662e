// X^T Y Gram matrix and Cholesky-QR (eigensolver/MultTm.h:33-53), FP64.
#ifndef TTDFT_MULTTM_H_
#define TTDFT_MULTTM_H_

#include <vector>

#include "petsc_shim.h"

class MultTM {
 public:
  MultTM() = default;
  // result = X^T Y, k x k column-major, resized by the callee (MultTm.cu:138).
  void mult(Mat& X, Mat& Y, std::vector<double>& result);
  // X <- X L^-T with X^T X = L L^T; throws ttdft::Error(TTG_NOT_SPD).
  void orth(Mat& X);
  virtual ~MultTM() = default;
};

#endif
