// Chebyshev filter over the device operator (eigensolver/ChebyShevFilter.h:29-40).
#ifndef TTDFT_CHEBYSHEVFILTER_H_
#define TTDFT_CHEBYSHEVFILTER_H_

#include "Mult.h"
#include "ProjectHamiltonianSparse.h"

class ChebyShevFilter {
 public:
  // Default schedule: FP64 throughout and the reference's degree m-1 result.
  ChebyShevFilter() : sched_{TTG_PREC_FP64, TTG_PREC_FP64, 0, 1} {}
  explicit ChebyShevFilter(ttg_sched s) : sched_(s) {}
  void computeFilteredSubspace(ProjectHamiltonianSparse& H, AX& ax, Mat& X, int basisSize, int m,
                               double a, double b, double a0, int num_X_blocks);
  void set_schedule(ttg_sched s) { sched_ = s; }

 private:
  ttg_sched sched_;
};

#endif
