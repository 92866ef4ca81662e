// chfsi_driver: runs the ChFSI loop of the reference's main.cc (:987-1207)
// through the reference-shaped C++ classes (AX, ChebyShevFilter, MultTM,
// EigenSolver), reading the operator and the start block from a binary file.
//
//   chfsi_driver <in.bin> <out.bin> [fp64|fp32|mixed]
//
// in.bin (little-endian):  int64 n, nnz_h, nproj, nnz_c, k, m, passes, lanczos_iters
//                          double a_init
//                          int64 h_row_ptr[n+1]; int32 h_col[nnz_h]; double h_val[nnz_h]
//                          int64 c_row_ptr[nproj+1]; int32 c_col[nnz_c]; double c_val[nnz_c]
//                          double d[nproj]; double X0[n*k] (column-major)
// out.bin:                 double upper, lower, eigvals[k], X[n*k] (column-major, rotated)
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

#include "ttdft/ChebyShevFilter.h"
#include "ttdft/EigenSolver.h"
#include "ttdft/Mult.h"
#include "ttdft/MultTm.h"

template <typename T> static void rd(std::ifstream& f, T* p, size_t n) {
  f.read(reinterpret_cast<char*>(p), sizeof(T) * n);
  if (!f) throw std::runtime_error("short input file");
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin [fp64|fp32|mixed]\n", argv[0]);
    return 2;
  }
  try {
    std::ifstream f(argv[1], std::ios::binary);
    int64_t hdr[8];
    rd(f, hdr, 8);
    const int64_t n = hdr[0], nnz_h = hdr[1], nproj = hdr[2], nnz_c = hdr[3];
    const int k = (int)hdr[4], m = (int)hdr[5], passes = (int)hdr[6], lanczos = (int)hdr[7];
    double a_init;
    rd(f, &a_init, 1);
    std::vector<int64_t> hp(n + 1), cp(nproj + 1);
    std::vector<int32_t> hc(nnz_h), cc(nnz_c);
    std::vector<double> hv(nnz_h), cv(nnz_c), d(nproj), x0((size_t)(n * k));
    rd(f, hp.data(), n + 1);
    rd(f, hc.data(), nnz_h);
    rd(f, hv.data(), nnz_h);
    rd(f, cp.data(), nproj + 1);
    rd(f, cc.data(), nnz_c);
    rd(f, cv.data(), nnz_c);
    rd(f, d.data(), nproj);
    rd(f, x0.data(), n * k);

    ProjectHamiltonianSparse H;
    Mat Hloc = MatCreateAIJShim(n, n, hp.data(), hc.data(), hv.data());
    Mat C = MatCreateAIJShim(nproj, n, cp.data(), cc.data(), cv.data());
    H.set(Hloc, C, d);

    ttg_sched sched{TTG_PREC_FP64, TTG_PREC_FP64, 0, 1};
    const std::string mode = argc > 3 ? argv[3] : "fp64";
    if (mode == "fp32") sched = ttg_sched{TTG_PREC_FP32, TTG_PREC_FP32, 0, 0};
    if (mode == "mixed") sched = ttg_sched{TTG_PREC_BF16, TTG_PREC_FP32, m / 4, 0};

    AX ax(1, k);                                   // main.cc:1032-1034
    ax.setup_system(H);
    EigenSolver eigen;
    double upper, lower;                           // main.cc:987-1003
    eigen.computeUpperBoundWithLanczos(H, lanczos, upper, lower);
    double b = upper, a = a_init, a0 = lower;      // main.cc:1011-1014 (first SCF step)
    Mat X = MatCreateDenseShim(n, k, x0.data());
    ChebyShevFilter filter(sched);
    MultTM multtm;
    std::vector<double> w(k);
    Mat Q = MatCreateDenseShim(k, k, nullptr);
    for (int pass = 0; pass < passes; ++pass) {    // main.cc:1035-1180
      filter.computeFilteredSubspace(H, ax, X, (int)n, m, a, b, a0, 1);
      multtm.orth(X);
      Mat HP = MatCreateDenseShim(n, k, nullptr);
      ax.perform_ax(X, HP);
      std::vector<double> pthp;
      multtm.mult(X, HP, pthp);
      MatDestroy(&HP);
      Mat P = MatCreateDenseShim(k, k, pthp.data());
      eigen.computeEigenPairsSeq(P, k, k, w, Q, true);
      MatDestroy(&P);
      a0 = w[0];
      a = w[k - 1];
    }
    // rotation X <- X Q (main.cc:1186-1207)
    double* xh = MatDenseGetArray(X);
    double* qh = MatDenseGetArray(Q);
    std::vector<double> xr((size_t)(n * k), 0.0);
    ttg_block* blk = ttdft::device_block(X, ax.op());
    ttdft::check(ttg_rotate(ax.op(), blk, qh), "ttg_rotate");
    ttdft::mark_device_modified(X);
    xh = MatDenseGetArray(X);
    std::ofstream o(argv[2], std::ios::binary);
    o.write(reinterpret_cast<const char*>(&upper), 8);
    o.write(reinterpret_cast<const char*>(&lower), 8);
    o.write(reinterpret_cast<const char*>(w.data()), 8 * k);
    o.write(reinterpret_cast<const char*>(xh), 8 * n * k);
    MatDestroy(&X);
    MatDestroy(&Q);
    H.Destroy();
    MatDestroy(&Hloc);
    MatDestroy(&C);
    std::printf("chfsi_driver: %d passes, lowest %.12f, upper bound %.6f\n", passes, w[0], upper);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "chfsi_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
