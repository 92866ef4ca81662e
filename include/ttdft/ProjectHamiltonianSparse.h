// Operator holder with the public members the reference's eigensolver reads
// (dft/ProjectHamiltonianSparse.h:97): H_loc, C_nloc = diag(D) C and
// C_nloc_trans = C^T.  D is kept explicit so that the device operator can
// apply C^T D C without forming C_nloc_trans C_nloc.
#ifndef TTDFT_PROJECT_HAMILTONIAN_SPARSE_H_
#define TTDFT_PROJECT_HAMILTONIAN_SPARSE_H_

#include <vector>

#include "petsc_shim.h"

class ProjectHamiltonianSparse {
 public:
  Mat H_loc = nullptr;        // N x N, AIJ
  Mat C_nloc = nullptr;       // nproj x N, AIJ, rows scaled by D
  Mat C_nloc_trans = nullptr; // N x nproj, AIJ (= C^T)
  std::vector<double> D;      // projector couplings
  Mat C = nullptr;            // nproj x N, AIJ, unscaled
  int tucker_ranks[3] = {0, 0, 0};  // (rx, ry, rz) when known: enables 3-D row tiling

  // Takes H_loc, C (nproj x N) and D; builds C_nloc and C_nloc_trans.
  void set(Mat h_loc, Mat c, const std::vector<double>& d);
  void Destroy();
};

#endif
