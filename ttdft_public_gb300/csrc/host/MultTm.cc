// MultTM over the C ABI (include/ttdft/MultTm.h); MultTm.cu:86-224 (mult),
// :226-467 (orth).
#include "ttdft/MultTm.h"

#include "ttdft/Mult.h"

static ttg_op* op_for(Mat X) {
  if (X->dev) return ttdft::current_op();
  ttg_op* op = ttdft::current_op();
  if (!op) throw std::logic_error("MultTM: no device operator (set up an AX first)");
  return op;
}

void MultTM::mult(Mat& X, Mat& Y, std::vector<double>& result) {
  ttg_op* op = op_for(X);
  ttg_block* x = ttdft::device_block(X, op);
  ttg_block* y = ttdft::device_block(Y, op);
  result.assign((size_t)X->n * X->n, 0.0);
  ttdft::check(ttg_gram(op, x, y, result.data()), "ttg_gram");
}

void MultTM::orth(Mat& X) {
  ttg_op* op = op_for(X);
  ttg_block* x = ttdft::device_block(X, op);
  ttdft::check(ttg_chol_qr(op, x), "ttg_chol_qr");
  ttdft::mark_device_modified(X);
}
