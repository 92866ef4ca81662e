// Host operator producer: assembles the projected Kohn-Sham Hamiltonian H_loc
// in a separable (Tucker) basis as a truncated CSR matrix, and the nonlocal
// projector matrix C_nloc.
//
// Follows ProjectHamiltonianSparse::Create_Hloc
// (dft/ProjectHamiltonianSparse.cc:330-575): for row I = (xI, yI, zI) with
// I = xI + rx*(yI + ry*zI) (x fastest, :420-433) the entries are
//   0.5*(DX[xI,xJ] MY[yI,yJ] MZ[zI,zJ] + MX DY MZ + MX MY DZ)      (:480-491)
//   + sum_abc G_abc PX_a[xI,xJ] PY_b[yI,yJ] PZ_c[zI,zJ]             (:516-543)
// and only |h| > truncation is kept (:545-548).  The potential here is given
// in canonical (CP) form, sum_t c_t PX_t (x) PY_t (x) PZ_t, which is a Tucker
// form with a superdiagonal core; a dense Tucker core is expanded by the
// caller into this form.
//
// The assembly is row-parallel (OpenMP) and prunes terms whose 1-D factors
// cannot reach the truncation threshold, so that large operators assemble in
// seconds.  Host-only code: no CUDA, no torch.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cstdlib>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Sparse1D {
  // row-wise sparse copy of an r x r matrix (entries above a drop tolerance)
  std::vector<int64_t> ptr;
  std::vector<int> col;
  std::vector<double> val;
  std::vector<double> rowmax;
};

Sparse1D make_sparse(const double* m, int r, double drop) {
  Sparse1D s;
  s.ptr.assign(r + 1, 0);
  s.rowmax.assign(r, 0.0);
  double amax = 0.0;
  for (int i = 0; i < r * r; ++i) amax = std::max(amax, std::fabs(m[i]));
  double thr = drop * amax;
  for (int i = 0; i < r; ++i) {
    for (int j = 0; j < r; ++j) {
      double v = m[(int64_t)i * r + j];
      if (std::fabs(v) > thr) {
        s.col.push_back(j);
        s.val.push_back(v);
        s.rowmax[i] = std::max(s.rowmax[i], std::fabs(v));
      }
    }
    s.ptr[i + 1] = (int64_t)s.col.size();
  }
  return s;
}

// Scratch of one thread: a dense row accumulator, a second one for the
// pattern-only potential (when there is one) and a bit per column marking
// the touched ones, scanned in column order when the row is emitted (no
// sort), with the range of touched words.
struct RowScratch {
  std::vector<double> row, extra;
  std::vector<uint64_t> bits;
  int64_t wlo, whi;
  RowScratch(int64_t n, bool with_extra)
      : row(n, 0.0), extra(with_extra ? n : 0, 0.0), bits(n / 64 + 1, 0), wlo(n), whi(-1) {}
};

// Builds one row of H_loc: the kinetic and potential Kronecker sums, then
// the entries above the truncation in column order.  An optional second CP
// potential (npat terms) widens the pattern only: an entry is kept when its
// value, or its value with that potential added, exceeds the truncation, and
// the value stored leaves the second potential out.
struct RowBuilder {
  int rx, ry, rz;
  int64_t N;
  const Sparse1D *sMX, *sMY, *sMZ, *sDX, *sDY, *sDZ;
  const std::vector<Sparse1D>*sPX, *sPY, *sPZ;
  int nterm;
  const double* coef;
  const std::vector<Sparse1D>*sQX, *sQY, *sQZ;
  int npat;
  const double* pcoef;
  double truncation, prune;

  void row(int64_t I, RowScratch& s, std::vector<int>& out_cols,
           std::vector<double>& out_vals) const {
    std::vector<double>& row = s.row;
    std::vector<double>& extra = s.extra;
    std::vector<uint64_t>& bits = s.bits;
    auto touch = [&](int64_t J) {
      const int64_t w = J >> 6;
      bits[w] |= 1ull << (J & 63);
      s.wlo = std::min(s.wlo, w);
      s.whi = std::max(s.whi, w);
    };
    // columns J0..J1 (inclusive) at once: whole words where it can
    auto touch_range = [&](int64_t J0, int64_t J1) {
      const int64_t w0 = J0 >> 6, w1 = J1 >> 6;
      const uint64_t m0 = ~0ull << (J0 & 63), m1 = ~0ull >> (63 - (J1 & 63));
      if (w0 == w1) {
        bits[w0] |= m0 & m1;
      } else {
        bits[w0] |= m0;
        for (int64_t w = w0 + 1; w < w1; ++w) bits[w] = ~0ull;
        bits[w1] |= m1;
      }
      s.wlo = std::min(s.wlo, w0);
      s.whi = std::max(s.whi, w1);
    };
    auto add = [&](int64_t J, double v) {
      touch(J);
      row[J] += v;
    };
      const int xI = (int)(I % rx);
      const int yI = (int)((I / rx) % ry);
      const int zI = (int)(I / ((int64_t)rx * ry));
      // kinetic: 0.5*(DX MY MZ + MX DY MZ + MX MY DZ)
      const Sparse1D* A[3][3] = {{sDX, sMY, sMZ}, {sMX, sDY, sMZ}, {sMX, sMY, sDZ}};
      for (int term = 0; term < 3; ++term) {
        const Sparse1D &ax = *A[term][0], &ay = *A[term][1], &az = *A[term][2];
        for (int64_t pz = az.ptr[zI]; pz < az.ptr[zI + 1]; ++pz) {
          const int zJ = az.col[pz];
          const double vz = 0.5 * az.val[pz];
          // products that cannot reach the truncation are not formed
          if (std::fabs(vz) * ay.rowmax[yI] * ax.rowmax[xI] <= prune) continue;
          for (int64_t py = ay.ptr[yI]; py < ay.ptr[yI + 1]; ++py) {
            const int yJ = ay.col[py];
            const double vyz = vz * ay.val[py];
            if (std::fabs(vyz) * ax.rowmax[xI] <= prune) continue;
            const int64_t base = (int64_t)rx * (yJ + (int64_t)ry * zJ);
            for (int64_t px = ax.ptr[xI]; px < ax.ptr[xI + 1]; ++px)
              add(base + ax.col[px], vyz * ax.val[px]);
          }
        }
      }
      // potential: sum_t c_t PX_t PY_t PZ_t, into `acc`
      auto add_cp = [&](const std::vector<Sparse1D>& PX, const std::vector<Sparse1D>& PY,
                        const std::vector<Sparse1D>& PZ, int n, const double* c,
                        std::vector<double>& acc) {
        for (int t = 0; t < n; ++t) {
          const Sparse1D &px = PX[t], &py = PY[t], &pz = PZ[t];
          const double bound = std::fabs(c[t]) * px.rowmax[xI] * py.rowmax[yI] * pz.rowmax[zI];
          if (bound <= prune) continue;
          for (int64_t qz = pz.ptr[zI]; qz < pz.ptr[zI + 1]; ++qz) {
            const int zJ = pz.col[qz];
            const double wz = c[t] * pz.val[qz];
            if (std::fabs(wz) * py.rowmax[yI] * px.rowmax[xI] <= prune) continue;
            for (int64_t qy = py.ptr[yI]; qy < py.ptr[yI + 1]; ++qy) {
              const int yJ = py.col[qy];
              const double w = wz * py.val[qy];
              if (std::fabs(w) * px.rowmax[xI] <= prune) continue;
              const int64_t base = (int64_t)rx * (yJ + (int64_t)ry * zJ);
              const int64_t q0 = px.ptr[xI], q1 = px.ptr[xI + 1];
              if (q1 == q0) continue;
              const int* cx = px.col.data();
              const double* __restrict__ vx = px.val.data() + q0;
              const int64_t n = q1 - q0;
              if (cx[q1 - 1] - cx[q0] == n - 1) {          // a run of columns: axpy
                double* __restrict__ a = acc.data() + base + cx[q0];
                for (int64_t i = 0; i < n; ++i) a[i] += w * vx[i];
                touch_range(base + cx[q0], base + cx[q1 - 1]);
              } else {
                double* a = acc.data() + base;
                for (int64_t i = 0; i < n; ++i) {
                  a[cx[q0 + i]] += w * vx[i];
                  touch(base + cx[q0 + i]);
                }
              }
            }
          }
        }
      };
      add_cp(*sPX, *sPY, *sPZ, nterm, coef, row);
      if (npat > 0) add_cp(*sQX, *sQY, *sQZ, npat, pcoef, extra);
      for (int64_t w = s.wlo; w <= s.whi; ++w) {
        uint64_t word = bits[w];
        bits[w] = 0;
        while (word) {
          const int J = (int)(w * 64 + __builtin_ctzll(word));
          word &= word - 1;
          const double v = row[J];
          bool keep = std::fabs(v) > truncation;
          if (npat > 0) {
            keep = keep || std::fabs(v + extra[J]) > truncation;
            extra[J] = 0.0;
          }
          if (keep) {
            out_cols.push_back(J);
            out_vals.push_back(v);
          }
          row[J] = 0.0;
        }
      }
      s.wlo = N;
      s.whi = -1;
  }
};

std::vector<Sparse1D> sparse_terms(const double* P, int n, int r, double drop) {
  std::vector<Sparse1D> out(n);
  for (int t = 0; t < n; ++t) out[t] = make_sparse(P + (int64_t)t * r * r, r, drop);
  return out;
}

}  // namespace

extern "C" {

// Assemble H_loc.
//   r[3]            : Tucker basis ranks (rx, ry, rz)
//   MX,MY,MZ        : 1-D overlap matrices, row-major r x r
//   DX,DY,DZ        : 1-D stiffness matrices (int psi' psi'), row-major r x r
//   nterm, coef     : CP potential, coef[t]
//   PX,PY,PZ        : nterm x r x r potential overlap matrices (row-major)
//   truncation      : keep |h| > truncation
//   drop            : relative drop tolerance for pruning 1-D factors (1e-15 typ.)
// Two-phase API: call with vals == nullptr to get row_ptr (size N+1) filled,
// then call again with col/vals of size row_ptr[N].
// Returns 0 on success, negative on bad arguments.
int ttg_host_assemble_hloc(const int* r, const double* MX, const double* MY,
                           const double* MZ, const double* DX, const double* DY,
                           const double* DZ, int nterm, const double* coef,
                           const double* PX, const double* PY, const double* PZ,
                           double truncation, double drop, int64_t* row_ptr,
                           int* col, double* vals) {
  if (!r || r[0] <= 0 || r[1] <= 0 || r[2] <= 0 || nterm < 0 || !row_ptr) return -1;
  const int rx = r[0], ry = r[1], rz = r[2];
  const int64_t N = (int64_t)rx * ry * rz;
  Sparse1D sMX = make_sparse(MX, rx, drop), sMY = make_sparse(MY, ry, drop),
           sMZ = make_sparse(MZ, rz, drop);
  Sparse1D sDX = make_sparse(DX, rx, drop), sDY = make_sparse(DY, ry, drop),
           sDZ = make_sparse(DZ, rz, drop);
  std::vector<Sparse1D> sPX = sparse_terms(PX, nterm, rx, drop),
                        sPY = sparse_terms(PY, nterm, ry, drop),
                        sPZ = sparse_terms(PZ, nterm, rz, drop);
  const bool fill = (vals != nullptr);
  const double prune = truncation * 1e-6;
  RowBuilder rb{rx, ry, rz, N, &sMX, &sMY, &sMZ, &sDX, &sDY, &sDZ, &sPX, &sPY, &sPZ, nterm, coef,
                nullptr, nullptr, nullptr, 0, nullptr, truncation, prune};

#pragma omp parallel
  {
    RowScratch sc(N, false);
    std::vector<int> cols;
    std::vector<double> vs;
#pragma omp for schedule(dynamic, 64)
    for (int64_t I = 0; I < N; ++I) {
      cols.clear();
      vs.clear();
      rb.row(I, sc, cols, vs);
      if (fill) {
        std::copy(cols.begin(), cols.end(), col + row_ptr[I]);
        std::copy(vs.begin(), vs.end(), vals + row_ptr[I]);
      } else {
        row_ptr[I + 1] = (int64_t)cols.size();
      }
    }
  }
  if (!fill) {
    row_ptr[0] = 0;
    for (int64_t I = 0; I < N; ++I) row_ptr[I + 1] += row_ptr[I];
  }
  return 0;
}

}  // extern "C"

namespace {

// One-pass assembly: every row is built once, into per-chunk buffers, then
// copied into col_out / val_out (malloc'ed here, released with ttg_host_free).
int assemble_once(const int* r, const double* MX, const double* MY, const double* MZ,
                  const double* DX, const double* DY, const double* DZ, int nterm,
                  const double* coef, const double* PX, const double* PY, const double* PZ,
                  int npat, const double* pcoef, const double* QX, const double* QY,
                  const double* QZ, double truncation, double drop, int64_t* row_ptr,
                  int** col_out, double** val_out) {
  if (!r || r[0] <= 0 || r[1] <= 0 || r[2] <= 0 || nterm < 0 || npat < 0 || !row_ptr ||
      !col_out || !val_out)
    return -1;
  if (npat > 0 && (!pcoef || !QX || !QY || !QZ)) return -1;
  const int rx = r[0], ry = r[1], rz = r[2];
  const int64_t N = (int64_t)rx * ry * rz;
  Sparse1D sMX = make_sparse(MX, rx, drop), sMY = make_sparse(MY, ry, drop),
           sMZ = make_sparse(MZ, rz, drop);
  Sparse1D sDX = make_sparse(DX, rx, drop), sDY = make_sparse(DY, ry, drop),
           sDZ = make_sparse(DZ, rz, drop);
  std::vector<Sparse1D> sPX = sparse_terms(PX, nterm, rx, drop),
                        sPY = sparse_terms(PY, nterm, ry, drop),
                        sPZ = sparse_terms(PZ, nterm, rz, drop);
  std::vector<Sparse1D> sQX = sparse_terms(QX, npat, rx, drop),
                        sQY = sparse_terms(QY, npat, ry, drop),
                        sQZ = sparse_terms(QZ, npat, rz, drop);
  RowBuilder rb{rx, ry, rz, N, &sMX, &sMY, &sMZ, &sDX, &sDY, &sDZ, &sPX, &sPY, &sPZ, nterm, coef,
                &sQX, &sQY, &sQZ, npat, pcoef, truncation, truncation * 1e-6};
  const int64_t chunk = 256, nchunks = (N + chunk - 1) / chunk;
  std::vector<std::vector<int>> ccol(nchunks);
  std::vector<std::vector<double>> cval(nchunks);
#pragma omp parallel
  {
    RowScratch sc(N, npat > 0);
#pragma omp for schedule(dynamic, 1)
    for (int64_t c = 0; c < nchunks; ++c) {
      for (int64_t I = c * chunk; I < std::min(N, (c + 1) * chunk); ++I) {
        const size_t before = ccol[c].size();
        rb.row(I, sc, ccol[c], cval[c]);
        row_ptr[I + 1] = (int64_t)(ccol[c].size() - before);
      }
    }
  }
  row_ptr[0] = 0;
  for (int64_t I = 0; I < N; ++I) row_ptr[I + 1] += row_ptr[I];
  const int64_t nnz = row_ptr[N];
  int* col = static_cast<int*>(std::malloc(std::max<int64_t>(nnz, 1) * sizeof(int)));
  double* vals = static_cast<double*>(std::malloc(std::max<int64_t>(nnz, 1) * sizeof(double)));
  if (!col || !vals) {
    std::free(col);
    std::free(vals);
    return -2;
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t c = 0; c < nchunks; ++c) {
    const int64_t o = row_ptr[c * chunk];
    std::copy(ccol[c].begin(), ccol[c].end(), col + o);
    std::copy(cval[c].begin(), cval[c].end(), vals + o);
    std::vector<int>().swap(ccol[c]);
    std::vector<double>().swap(cval[c]);
  }
  *col_out = col;
  *val_out = vals;
  return 0;
}

}  // namespace

extern "C" {

// ttg_host_assemble_hloc in one pass (malloc'ed col_out / val_out, released
// with ttg_host_free).  row_ptr: N + 1 entries, filled.
int ttg_host_assemble_hloc_once(const int* r, const double* MX, const double* MY,
                                const double* MZ, const double* DX, const double* DY,
                                const double* DZ, int nterm, const double* coef,
                                const double* PX, const double* PY, const double* PZ,
                                double truncation, double drop, int64_t* row_ptr,
                                int** col_out, double** val_out) {
  return assemble_once(r, MX, MY, MZ, DX, DY, DZ, nterm, coef, PX, PY, PZ, 0, nullptr, nullptr,
                       nullptr, nullptr, truncation, drop, row_ptr, col_out, val_out);
}

// As ttg_host_assemble_hloc_once, with a second CP potential (npat terms:
// pcoef, QX, QY, QZ laid out like coef, PX, PY, PZ) that widens the pattern
// only: an entry is kept when |h| or |h + q| exceeds the truncation, q being
// the second potential's matrix entry, and the stored value is h.  A frozen
// pattern built this way also holds the entries that a later potential of
// that shape raises above the truncation.
int ttg_host_assemble_hloc_pattern(const int* r, const double* MX, const double* MY,
                                   const double* MZ, const double* DX, const double* DY,
                                   const double* DZ, int nterm, const double* coef,
                                   const double* PX, const double* PY, const double* PZ,
                                   int npat, const double* pcoef, const double* QX,
                                   const double* QY, const double* QZ, double truncation,
                                   double drop, int64_t* row_ptr, int** col_out,
                                   double** val_out) {
  return assemble_once(r, MX, MY, MZ, DX, DY, DZ, nterm, coef, PX, PY, PZ, npat, pcoef, QX, QY,
                       QZ, truncation, drop, row_ptr, col_out, val_out);
}

void ttg_host_free(void* p) { std::free(p); }

// Separable nonlocal projector matrix C (nproj x N, CSR):
//   C[a, J] = cx[a, xJ] * cy[a, yJ] * cz[a, zJ], kept where |C| > tol.
// Follows ProjectHamiltonianSparse::Create_Cnloc
// (dft/ProjectHamiltonianSparse.cc:83-328) for projectors whose Tucker form is
// rank one.  Two-phase like ttg_host_assemble_hloc.
int ttg_host_assemble_cnloc(const int* r, int nproj, const double* cx,
                            const double* cy, const double* cz, double tol,
                            int64_t* row_ptr, int* col, double* vals) {
  if (!r || nproj < 0 || !row_ptr) return -1;
  const int rx = r[0], ry = r[1], rz = r[2];
  const bool fill = (vals != nullptr);
  row_ptr[0] = 0;
  for (int a = 0; a < nproj; ++a) {
    int64_t out = fill ? row_ptr[a] : 0;
    int64_t cnt = 0;
    for (int zJ = 0; zJ < rz; ++zJ)
      for (int yJ = 0; yJ < ry; ++yJ) {
        const double wyz = cy[(int64_t)a * ry + yJ] * cz[(int64_t)a * rz + zJ];
        for (int xJ = 0; xJ < rx; ++xJ) {
          const double v = wyz * cx[(int64_t)a * rx + xJ];
          if (std::fabs(v) > tol) {
            if (fill) {
              col[out] = xJ + rx * (yJ + ry * zJ);
              vals[out] = v;
              ++out;
            }
            ++cnt;
          }
        }
      }
    if (!fill) row_ptr[a + 1] = row_ptr[a] + cnt;
  }
  return 0;
}

}  // extern "C"
