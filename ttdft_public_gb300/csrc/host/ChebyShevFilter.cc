// ChebyShevFilter::computeFilteredSubspace (include/ttdft/ChebyShevFilter.h)
// over the C ABI.  The reference splits X into num_X_blocks column chunks to
// bound host memory (eigensolver/ChebyShevFilter.cc:57-61); the device
// filter handles the whole block in one pass per degree, so the chunks only
// bound the block width here.
#include "ttdft/ChebyShevFilter.h"

void ChebyShevFilter::computeFilteredSubspace(ProjectHamiltonianSparse& H, AX& ax, Mat& X,
                                              int basisSize, int m, double a, double b, double a0,
                                              int num_X_blocks) {
  (void)H;
  (void)num_X_blocks;
  if (!ax.op()) throw std::logic_error("ChebyShevFilter: AX not set up");
  if (X->m != basisSize) throw std::invalid_argument("ChebyShevFilter: basisSize");
  ttg_block* x = ttdft::device_block(X, ax.op());
  ttdft::check(ttg_cheb_filter(ax.op(), x, m, a, b, a0, sched_), "ttg_cheb_filter");
  ttdft::mark_device_modified(X);
}
