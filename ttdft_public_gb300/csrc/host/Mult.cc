// AX over the C ABI (include/ttdft/Mult.h).  Follows the lifetime of the
// reference's AX (eigensolver/MultCuda.cu:38-103 ctor, :105-371 setup,
// :719-820 perform_ax, :673-717 free), with the result actually stored into
// the caller's AX (the reference drops it, MultCuda.cu:781-820).
#include "ttdft/Mult.h"

namespace {
ttg_op* g_current = nullptr;
}

namespace ttdft {
ttg_op* current_op() { return g_current; }
void set_current_op(ttg_op* op) { g_current = op; }
}  // namespace ttdft

AX::AX(int num_bg, int num_wfns) : num_wfns_(num_wfns) {
  if (num_bg != 1) throw std::invalid_argument("one GPU: num_bg must be 1");
}

void AX::setup_system(Mat A) {
  ProjectHamiltonianSparse H;
  H.H_loc = A;
  setup_system(H);
}

void AX::setup_system(ProjectHamiltonianSparse& H) {
  free_mata_on_device();
  Mat A = H.H_loc;
  if (!A || A->kind != _p_Mat::AIJ || A->m != A->n) throw std::invalid_argument("H_loc: square AIJ");
  const int32_t nproj = H.C ? (int32_t)H.C->m : 0;
  const bool tucker = H.tucker_ranks[0] > 0;
  ttdft::check(ttg_op_create_tucker(A->m, A->row_ptr.data(), A->col.data(), A->val.data(), nproj,
                                    nproj ? H.C->row_ptr.data() : nullptr,
                                    nproj ? H.C->col.data() : nullptr,
                                    nproj ? H.C->val.data() : nullptr,
                                    nproj ? H.D.data() : nullptr,
                                    tucker ? H.tucker_ranks : nullptr, num_wfns_, &op_),
               "ttg_op_create_tucker");
  ttdft::set_current_op(op_);
}

void AX::perform_ax(Mat& X, Mat& AXm) {
  if (!op_) throw std::logic_error("AX::perform_ax before setup_system");
  if (X->m != AXm->m || X->n != AXm->n) throw std::invalid_argument("AX shape");
  ttg_block* x = ttdft::device_block(X, op_);
  ttg_block* y = ttdft::device_block(AXm, op_);
  ttdft::check(ttg_apply_h(op_, x, y), "ttg_apply_h");
  ttdft::mark_device_modified(AXm);
}

void AX::free_mata_on_device() {
  if (op_) {
    if (ttdft::current_op() == op_) ttdft::set_current_op(nullptr);
    ttg_op_destroy(op_);
    op_ = nullptr;
  }
}

AX::~AX() { free_mata_on_device(); }
