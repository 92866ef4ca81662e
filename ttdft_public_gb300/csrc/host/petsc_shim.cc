// Single-rank Mat shim (see include/ttdft/petsc_shim.h) and the operator
// holder of include/ttdft/ProjectHamiltonianSparse.h.
#include "ttdft/petsc_shim.h"

#include <algorithm>
#include <cstring>

#include "ttdft/ProjectHamiltonianSparse.h"

Mat MatCreateDenseShim(int64_t m, int64_t n, const double* data) {
  Mat A = new _p_Mat();
  A->kind = _p_Mat::DENSE;
  A->m = m;
  A->n = n;
  A->data.assign((size_t)(m * n), 0.0);
  if (data) std::memcpy(A->data.data(), data, sizeof(double) * m * n);
  return A;
}

Mat MatCreateAIJShim(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col,
                     const double* val) {
  Mat A = new _p_Mat();
  A->kind = _p_Mat::AIJ;
  A->m = m;
  A->n = n;
  A->row_ptr.assign(row_ptr, row_ptr + m + 1);
  A->col.assign(col, col + row_ptr[m]);
  A->val.assign(val, val + row_ptr[m]);
  return A;
}

void MatGetSize(Mat A, int64_t* m, int64_t* n) {
  if (m) *m = A->m;
  if (n) *n = A->n;
}

double* MatDenseGetArray(Mat A) {
  if (A->kind != _p_Mat::DENSE) throw std::invalid_argument("MatDenseGetArray on a sparse Mat");
  if (!A->host_valid && A->dev) {
    ttdft::check(ttg_block_get(A->dev, A->data.data(), A->m), "ttg_block_get");
    A->host_valid = true;
  }
  return A->data.data();
}

void MatDenseRestoreArray(Mat A) {
  A->host_valid = true;
  A->dev_valid = false;
}

void MatDestroy(Mat* A) {
  if (!A || !*A) return;
  if ((*A)->dev) ttg_block_destroy((*A)->dev);
  delete *A;
  *A = nullptr;
}

namespace ttdft {

ttg_block* device_block(Mat A, ttg_op* op) {
  if (!A || A->kind != _p_Mat::DENSE) throw std::invalid_argument("dense Mat expected");
  if (!op) throw std::invalid_argument("no device operator: call AX::setup_system first");
  if (A->dev && !A->dev_valid) {
    // stale device copy: refresh from the host
  }
  if (!A->dev) {
    check(ttg_block_create(op, (int32_t)A->n, &A->dev), "ttg_block_create");
    A->dev_valid = false;
  }
  if (!A->dev_valid) {
    check(ttg_block_set(A->dev, A->data.data(), A->m), "ttg_block_set");
    A->dev_valid = true;
  }
  return A->dev;
}

void mark_device_modified(Mat A) {
  A->dev_valid = true;
  A->host_valid = false;
}

}  // namespace ttdft

static Mat transpose_aij(Mat A) {
  std::vector<int64_t> rp(A->n + 1, 0);
  for (int64_t e = 0; e < A->row_ptr[A->m]; ++e) rp[A->col[e] + 1]++;
  for (int64_t j = 0; j < A->n; ++j) rp[j + 1] += rp[j];
  std::vector<int32_t> col(A->row_ptr[A->m]);
  std::vector<double> val(A->row_ptr[A->m]);
  std::vector<int64_t> pos(rp.begin(), rp.end() - 1);
  for (int64_t i = 0; i < A->m; ++i)
    for (int64_t e = A->row_ptr[i]; e < A->row_ptr[i + 1]; ++e) {
      const int64_t j = A->col[e];
      col[pos[j]] = (int32_t)i;
      val[pos[j]] = A->val[e];
      pos[j]++;
    }
  return MatCreateAIJShim(A->n, A->m, rp.data(), col.data(), val.data());
}

void ProjectHamiltonianSparse::set(Mat h_loc, Mat c, const std::vector<double>& d) {
  H_loc = h_loc;
  C = c;
  D = d;
  if (c && c->m > 0) {
    std::vector<double> sv(c->val);
    for (int64_t a = 0; a < c->m; ++a)
      for (int64_t e = c->row_ptr[a]; e < c->row_ptr[a + 1]; ++e) sv[e] *= d[a];
    C_nloc = MatCreateAIJShim(c->m, c->n, c->row_ptr.data(), c->col.data(), sv.data());
    C_nloc_trans = transpose_aij(c);
  }
}

void ProjectHamiltonianSparse::Destroy() {
  MatDestroy(&C_nloc);
  MatDestroy(&C_nloc_trans);
}
