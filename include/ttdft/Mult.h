// AX: device copy of the projected Hamiltonian and the product A*X.
// Same class, constructor and method names as the reference
// (eigensolver/Mult.h:30-61).  One GPU: num_bg must be 1.
#ifndef TTDFT_MULT_H_
#define TTDFT_MULT_H_

#include "ProjectHamiltonianSparse.h"
#include "petsc_shim.h"

class AX {
 public:
  AX(int num_bg, int num_wfns);
  // H_loc only (the reference's signature, MultCuda.cu:105-206).
  void setup_system(Mat A);
  // H_loc plus the nonlocal C^T D C, applied inside the same launches.
  void setup_system(ProjectHamiltonianSparse& H);
  // AX = H X (FP64).  AX must be pre-allocated by the caller (Mult.h:49-51).
  void perform_ax(Mat& X, Mat& AXm);
  void free_mata_on_device();
  ~AX();

  ttg_op* op() const { return op_; }

 private:
  int num_wfns_;
  ttg_op* op_ = nullptr;
};

namespace ttdft {
// The operator that MultTM and EigenSolver use when they are not handed one
// (the last AX that was set up; one process drives one GPU).
ttg_op* current_op();
void set_current_op(ttg_op* op);
}  // namespace ttdft

#endif
