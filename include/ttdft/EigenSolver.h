// Dense subspace eigensolve and Lanczos spectral bounds
// (eigensolver/EigenSolver.h:30-45), computed on the GPU in FP64.
#ifndef TTDFT_EIGENSOLVER_H_
#define TTDFT_EIGENSOLVER_H_

#include <cstdint>
#include <vector>

#include "ProjectHamiltonianSparse.h"
#include "petsc_shim.h"

class EigenSolver {
 public:
  // Ascending eigenvalues into eigVals (pre-sized by the caller), eigenvectors
  // as columns of eigMat (dense, numGlobalRows x numberEigenPairs).  `lapack`
  // is accepted for signature compatibility.
  void computeEigenPairsSeq(Mat& A, int numberEigenPairs, int numGlobalRows,
                            std::vector<double>& eigVals, Mat& eigMat, bool lapack);
  // upper = |lambda_max(T)| + |f|, lower = lambda_min(T).  The start vector is
  // uniform random in [0,1) from `seed` (the reference uses VecSetRandom).
  void computeUpperBoundWithLanczos(ProjectHamiltonianSparse& H, int maxLanczosIteration,
                                    double& upperBound, double& lowerBound);
  uint64_t seed = 12345;
};

#endif
