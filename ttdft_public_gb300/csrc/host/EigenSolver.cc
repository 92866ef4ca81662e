// EigenSolver over the C ABI (include/ttdft/EigenSolver.h);
// EigenSolver.cc:30-184 (dense eig), :186-388 (Lanczos bounds).
#include "ttdft/EigenSolver.h"

#include <random>

#include "ttdft/Mult.h"

void EigenSolver::computeEigenPairsSeq(Mat& A, int numberEigenPairs, int numGlobalRows,
                                       std::vector<double>& eigVals, Mat& eigMat, bool lapack) {
  (void)lapack;
  ttg_op* op = ttdft::current_op();
  if (!op) throw std::logic_error("EigenSolver: no device operator (set up an AX first)");
  const int k = numberEigenPairs;
  if (A->m != numGlobalRows || A->n != numGlobalRows || k != numGlobalRows)
    throw std::invalid_argument("computeEigenPairsSeq: all eigenpairs of a square matrix");
  std::vector<double> w(k);
  double* a = MatDenseGetArray(A);
  double* v = MatDenseGetArray(eigMat);
  ttdft::check(ttg_syev(op, k, a, w.data(), v), "ttg_syev");
  MatDenseRestoreArray(eigMat);
  if ((int)eigVals.size() < k) eigVals.resize(k);
  for (int i = 0; i < k; ++i) eigVals[i] = w[i];
}

void EigenSolver::computeUpperBoundWithLanczos(ProjectHamiltonianSparse& H, int maxLanczosIteration,
                                               double& upperBound, double& lowerBound) {
  ttg_op* op = ttdft::current_op();
  AX* own = nullptr;
  if (!op) {
    own = new AX(1, 1);
    own->setup_system(H);
    op = own->op();
  }
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::vector<double> v0((size_t)H.H_loc->m);
  for (auto& x : v0) x = u(rng);
  ttg_status s = ttg_lanczos_bounds(op, v0.data(), maxLanczosIteration, &upperBound, &lowerBound);
  delete own;
  ttdft::check(s, "ttg_lanczos_bounds");
}
