// Minimal single-rank stand-in for the PETSc Mat handle that the reference's
// eigensolver classes take (PETSc itself is not available here).  A Mat is
// either dense (N x k, column-major, like MATDENSE) or sparse CSR (like
// MATAIJ).  A dense Mat can carry a device-resident copy (a ttg_block) so
// that consecutive calls (filter -> orth -> Rayleigh-Ritz) stay on the GPU;
// the host copy is refreshed only when it is read.
#ifndef TTDFT_PETSC_SHIM_H_
#define TTDFT_PETSC_SHIM_H_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ttg.h"

namespace ttdft {

// Raised instead of the reference's std::terminate(): carries the ttg status.
class Error : public std::runtime_error {
 public:
  Error(ttg_status s, const std::string& what)
      : std::runtime_error(what + ": " + ttg_status_string(s)), status(s) {}
  ttg_status status;
};

inline void check(ttg_status s, const char* what) {
  if (s != TTG_OK) throw Error(s, what);
}

}  // namespace ttdft

struct _p_Mat {
  enum Kind { DENSE, AIJ } kind = DENSE;
  int64_t m = 0, n = 0;
  // dense: column-major m x n
  std::vector<double> data;
  // sparse CSR
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col;
  std::vector<double> val;
  // device copy of a dense Mat (owned), and which side is current
  ttg_block* dev = nullptr;
  bool host_valid = true;
  bool dev_valid = false;
};
typedef _p_Mat* Mat;

// Creation / access, named after the PETSc calls the reference makes.
Mat MatCreateDenseShim(int64_t m, int64_t n, const double* data /* may be null */);
Mat MatCreateAIJShim(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col,
                     const double* val);
void MatGetSize(Mat A, int64_t* m, int64_t* n);
// Host pointer to the (current) column-major data of a dense Mat.
double* MatDenseGetArray(Mat A);
// Marks the host data as modified (device copy stale).
void MatDenseRestoreArray(Mat A);
void MatDestroy(Mat* A);

namespace ttdft {
// Device block of a dense Mat for `op`, uploading the host data if needed.
ttg_block* device_block(Mat A, ttg_op* op);
// After a device-side update of A's block.
void mark_device_modified(Mat A);
}  // namespace ttdft

#endif  // TTDFT_PETSC_SHIM_H_
