/*
 * ttg.h -- C ABI of the GB300 (sm_103a) Chebyshev-filtered subspace
 * iteration library (libttg.so).
 *
 * Plain C types only: pointers, sizes, doubles.  Every entry point returns a
 * ttg_status; nothing terminates the process.  One CUDA stream per ttg_op;
 * calls on one handle are not thread-safe, calls on different handles are.
 * Entry points that return data in host memory synchronise the op's stream;
 * the others only enqueue work.  The library's streams are blocking streams:
 * work the caller enqueued on the legacy default stream before a call (for
 * example filling an input buffer) completes before the call's kernels run.
 *
 * Layout conventions (those of the reference's PETSc dense Mats):
 *   - a vector block X is N x k, column-major (one column per state), ld >= N;
 *   - k x k matrices (overlap, projected H, eigenvectors) are column-major;
 *   - CSR matrices use int64 row pointers and int32 column indices.
 * Inside the library, blocks live in HBM row-major (one row per basis index)
 * so that a row of X is one contiguous, vector-loadable segment.
 */
#ifndef TTG_H_
#define TTG_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TTG_OK = 0,
  TTG_BAD_ARG = 1,     /* null pointer, size out of range, mismatched shapes */
  TTG_BAD_CSR = 2,     /* row pointers not monotone, column out of range, ... */
  TTG_OOM = 3,         /* device allocation failed */
  TTG_NOT_SPD = 4,     /* Cholesky met a non-positive pivot */
  TTG_NONFINITE = 5,   /* NaN/Inf found in an input or an intermediate */
  TTG_TIMEOUT = 6,     /* a bounded device-side wait ran out */
  TTG_CUDA_ERR = 7,    /* a CUDA runtime call failed */
  TTG_NO_DEVICE = 8,   /* no usable sm_100+ device */
  TTG_NOT_CONVERGED = 9 /* an iteration hit its limit (eigensolver, Fermi) */
} ttg_status;

typedef enum {
  TTG_PREC_FP64 = 0,   /* H and the block in FP64, FP64 accumulation */
  TTG_PREC_FP32 = 1,   /* H and the block in FP32, FP32 accumulation */
  TTG_PREC_BF16 = 2,   /* H and the block stored in BF16, FP32 accumulation */
  TTG_PREC_DF64 = 3    /* FP64 values as pairs of FP32 (~47 bits) on the FP32 pipes */
} ttg_prec;

/* Precision schedule of one Chebyshev filter call: the first `n_low` degrees
 * run in `low`, the remaining ones in `high`.  `return_prev` = 1 reproduces
 * the reference exactly: its filter hands back the degree m-1 iterate
 * (eigensolver/ChebyShevFilter.cc:163-176), which this library computes
 * with m-1 operator applications; 0 returns the degree-m iterate. */
typedef struct {
  int32_t low;
  int32_t high;
  int32_t n_low;
  int32_t return_prev;
} ttg_sched;

typedef struct ttg_op ttg_op;        /* device-resident operator + workspace */
typedef struct ttg_block ttg_block;  /* device-resident N x k FP64 block */

typedef struct {
  int64_t n;              /* rows of H_loc */
  int64_t nnz_h;          /* nonzeros of H_loc */
  int64_t nnz_c;          /* nonzeros of C */
  int32_t nproj;          /* projector rows of C */
  int32_t group_rows;     /* rows per row group of the device format */
  int64_t n_groups;
  int64_t stored_cols;    /* merged column slots over all groups */
  double fill;            /* (nnz_h + nnz_c^T) / (group_rows * stored_cols) */
  int64_t device_bytes;   /* HBM held by the operator */
  int64_t launches;       /* kernels this op has launched so far */
  int64_t n_tiles;        /* 64-row tiles of the tensor-core format (0: none) */
  int64_t tile_slots;     /* merged column slots over all tiles */
  double tile_fill;       /* (nnz_h + nnz_c^T) / (64 * tile_slots) */
  int64_t umma_tiles;     /* 128-row tiles of the tcgen05 format (0: none) */
  int64_t umma_slots;     /* merged column slots over those tiles */
  int64_t shifted_orth;   /* shifted Cholesky-QR steps ttg_chfsi_pass needed so far */
} ttg_op_info_t;

/* ---- device and operator ------------------------------------------------ */

/* Library version string and the device it would use. */
const char* ttg_version(void);
ttg_status ttg_device_query(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);
const char* ttg_status_string(ttg_status s);
/* Number of kernels this library has launched in the process so far (all
 * entry points, all operators).  No counterpart in the reference. */
int64_t ttg_kernel_launches(void);

/* Upload the projected Hamiltonian.  Replaces AX::AX + AX::setup_system +
 * AX::setup_mata_on_device (eigensolver/Mult.h:37-44,
 * eigensolver/MultCuda.cu:38-371), which copy H_loc to the device, and
 * takes the nonlocal part that ChebyShevFilter applies with PETSc on the host
 * (eigensolver/ChebyShevFilter.cc:103-124; matrices from
 * dft/ProjectHamiltonianSparse.h:97): C (nproj x n) and D (nproj) such that
 * C_nloc = diag(D) C and C_nloc_trans = C^T.  nproj may be 0.
 * max_k bounds the block width used with this op.  The CSR is validated on
 * the host before anything is launched (TTG_BAD_CSR). */
ttg_status ttg_op_create(int64_t n, const int64_t* h_row_ptr, const int32_t* h_col,
                         const double* h_val, int32_t nproj, const int64_t* c_row_ptr,
                         const int32_t* c_col, const double* c_val, const double* d,
                         int32_t max_k, ttg_op** out);
/* As ttg_op_create, for an H_loc in a separable basis of Tucker ranks
 * (rx, ry, rz), rows ordered I = x + rx*(y + ry*z) as Create_Hloc orders
 * them (dft/ProjectHamiltonianSparse.cc:420-433).  The ranks let the library
 * tile rows in 4 x 4 x 4 blocks for the tensor-core SpMM; NULL gives tiles of
 * consecutive rows. */
ttg_status ttg_op_create_tucker(int64_t n, const int64_t* h_row_ptr, const int32_t* h_col,
                                const double* h_val, int32_t nproj, const int64_t* c_row_ptr,
                                const int32_t* c_col, const double* c_val, const double* d,
                                const int32_t* tucker_ranks, int32_t max_k, ttg_op** out);
/* Arithmetic of the H X product inside ttg_rayleigh_ritz / ttg_chfsi_pass:
 * TTG_PREC_DF64 (default: FP64-level accuracy at the FP32 rate) or
 * TTG_PREC_FP64 (native FP64, the reference's arithmetic). */
ttg_status ttg_op_set_rr_precision(ttg_op* op, int32_t prec);
/* Replaces AX::free_mata_on_device / AX::~AX (eigensolver/MultCuda.cu:673-717). */
ttg_status ttg_op_destroy(ttg_op* op);
ttg_status ttg_op_info(const ttg_op* op, ttg_op_info_t* info);
/* The op's cudaStream_t, as an opaque pointer, for callers that overlap work. */
void* ttg_op_stream(ttg_op* op);
/* Waits for the op's stream; TTG_TIMEOUT if a bounded wait inside a
 * tensor-memory filter kernel ran out since the last check. */
ttg_status ttg_op_sync(ttg_op* op);
/* Device-side timing on the op's stream (slot 0..15). */
ttg_status ttg_op_record(ttg_op* op, int32_t slot);
ttg_status ttg_op_elapsed_ms(ttg_op* op, int32_t slot0, int32_t slot1, float* ms);

/* Device time of the fused filter-degree kernels (one launch per degree, or
 * per 256-column block of wider blocks) and of the other stages of a ChFSI
 * pass and an SCF iteration, by kind.  With timing on, each such launch (or
 * stage) is bracketed by two CUDA events on the operator's stream; the pairs
 * are read back in batches
 * (no host wait per launch).  ttg_op_kernel_time synchronises the stream and
 * returns the total milliseconds and the launch count of one kind since
 * timing was switched on; enable = 0 switches it off and clears the totals. */
#define TTG_KT_UMMA_FP32 0   /* tcgen05 FP32 degree (three-term BF16 split) */
#define TTG_KT_TC_FP32 1     /* mma.sync FP32 degree (3xTF32) */
#define TTG_KT_TC_BF16 2     /* mma.sync BF16 degree */
#define TTG_KT_ROWGROUP 3    /* CUDA-core row-group degree (any precision) */
#define TTG_KT_UMMA_BF16 4   /* tcgen05 BF16 degree */
#define TTG_KT_HARTREE 5     /* ttg_hartree_device: factors + three tcgen05 contractions */
#define TTG_KT_DENSITY 6     /* ttg_density_device: mode products + squared sum */
#define TTG_KT_ORTH_GRAM 7   /* ttg_chfsi_pass orthonormalisation: X^T X */
#define TTG_KT_ORTH_CHOL 8   /*   Cholesky and L^-1 (k x k) */
#define TTG_KT_ORTH_UPDATE 9 /*   X <- X L^-T */
#define TTG_KT_RR_HX 10      /* Rayleigh-Ritz: H X */
#define TTG_KT_RR_GRAM 11    /*   X^T (H X) */
#define TTG_KT_RR_EIG 12     /*   k x k eigensolve */
#define TTG_KT_RR_ROTATE 13  /*   X <- X Q */
#define TTG_KT_KINDS 14
ttg_status ttg_op_kernel_timing(ttg_op* op, int32_t enable);
ttg_status ttg_op_kernel_time(ttg_op* op, int32_t kind, double* ms_total, int64_t* launches);

/* ---- vector blocks (the reference's dense Mat X, N x k) ----------------- */

ttg_status ttg_block_create(ttg_op* op, int32_t k, ttg_block** out);
ttg_status ttg_block_destroy(ttg_block* b);
int32_t ttg_block_cols(const ttg_block* b);
/* Host <-> device, column-major N x k with leading dimension ld. */
ttg_status ttg_block_set(ttg_block* b, const double* x_colmajor, int64_t ld);
ttg_status ttg_block_get(ttg_block* b, double* x_colmajor, int64_t ld);
/* Device-pointer variants (no host copy); column-major, ld >= N. */
ttg_status ttg_block_set_device(ttg_block* b, const double* x_colmajor_dev, int64_t ld);
ttg_status ttg_block_get_device(ttg_block* b, double* x_colmajor_dev, int64_t ld);
ttg_status ttg_block_copy(ttg_block* dst, const ttg_block* src);

/* ---- the hot path --------------------------------------------------------- */

/* Chebyshev filter, in place on X.  Replaces
 * ChebyShevFilter::computeFilteredSubspace (eigensolver/ChebyShevFilter.h:31-39,
 * eigensolver/ChebyShevFilter.cc:34-189): a = lower bound of the unwanted
 * spectrum, b = upper bound, a0 = lowest wanted eigenvalue, m = degree.
 * Each degree is one fused launch: Ynew = alpha*(H_loc Y + C^T D C Y)
 * + beta*Y + delta*X.  num_x_blocks of the reference only splits the columns
 * to bound host memory; here the whole block is filtered at once. */
ttg_status ttg_cheb_filter(ttg_op* op, ttg_block* X, int32_t m, double a, double b,
                           double a0, ttg_sched sched);

/* HX = (H_loc + C^T D C) X in FP64.  Replaces AX::perform_ax
 * (eigensolver/Mult.h:46-53, eigensolver/MultCuda.cu:719-820) plus the
 * nonlocal MatMatMults of main.cc:1066-1092. */
ttg_status ttg_apply_h(ttg_op* op, const ttg_block* X, ttg_block* HX);

/* S = X^T Y (k x k, column-major).  Replaces MultTM::mult
 * (eigensolver/MultTm.h:37, eigensolver/MultTm.cu:86-224).  FP64 data and
 * result, computed on the tensor cores: each value becomes six exact BF16
 * digits on a power-of-two scale of its row, the digit products are summed
 * exactly in tensor memory and the 96-deep groups in double-FP32, so an entry
 * lands within about 2^-48 of the product of its two rows' scales times the
 * length (measured: within 2^-44 of the sum of |terms|).  When an operand's
 * alignment rules the tensor cores out, the products and sums run in
 * double-FP32 on the CUDA cores (each value a pair of floats, about 47
 * significant bits, FP32 exponent range; within ~6e-14 of the sum of |terms|).
 * s_host may be NULL when only the device copy is wanted (kept inside the
 * op). */
ttg_status ttg_gram(ttg_op* op, const ttg_block* X, const ttg_block* Y, double* s_host);

/* S = X^T Y like ttg_gram, for callers that cannot allocate device memory
 * (memory-pool or arena owners, plugins whose host forbids cudaMalloc after
 * start-up, code that must not synchronise the device).  No counterpart in
 * the reference.  X and Y are device pointers, row-major n x k with leading
 * dimension ld; S is a device pointer, k x k column-major; stream may be NULL.
 * Allocates nothing: the split-row partial sums live in a fixed 16 MiB
 * __device__ array that every GPU loading this library holds until exit, so
 * k*k must not exceed 2,097,152 (k <= 1448), else TTG_BAD_ARG.  Arithmetic:
 * double-FP32 (about 47 bits), the fallback path of ttg_gram.  The first call on a device looks up
 * the array's address (with lazy module loading this also loads the library's
 * device code and commits the array), so make it at start-up, before any
 * stream capture and before the host's no-allocation phase begins.  The
 * address is cached per device for the life of the process: after a
 * cudaDeviceReset of that device, do not call this entry point on it again.
 * All calls share the array: calls that overlap on the GPU race. */
ttg_status ttg_gram_noalloc(const double* x_dev, const double* y_dev, int64_t n, int32_t k,
                            int64_t ld, double* s_dev, void* stream);

/* Cholesky-QR: S = X^T X = L L^T, X <- X L^-T.  Replaces MultTM::orth
 * (eigensolver/MultTm.h:39, eigensolver/MultTm.cu:226-467).  The Gram matrix
 * S and the product X L^-T run as ttg_gram does (tensor cores, about 2^-48
 * relative to the row scales; X L^-T also scales X's columns to powers of two
 * first, since L^-T undoes them); the Cholesky factorisation and L^-1 are
 * FP64 (blocked on many CTAs for k > 128).  Orthogonality degrades with
 * cond(X)^2 times the Gram's relative error, a few times sooner than with
 * native FP64.
 * Returns TTG_NOT_SPD (X untouched) when S is not numerically positive
 * definite. */
ttg_status ttg_chol_qr(ttg_op* op, ttg_block* X);

/* Symmetric eigendecomposition of a k x k column-major FP64 matrix, ascending
 * eigenvalues, eigenvectors as columns.  Replaces
 * EigenSolver::computeEigenPairsSeq (eigensolver/EigenSolver.h:32-38,
 * eigensolver/EigenSolver.cc:30-184).  Host in/out; the work runs on the GPU. */
ttg_status ttg_syev(ttg_op* op, int32_t k, const double* a_host, double* w_host,
                    double* v_host);

/* Rayleigh-Ritz on X: HX = H X, P = X^T HX, P = Q diag(w) Q^T; if rotate != 0
 * also X <- X Q.  main.cc:1066-1115 (projection + eig) and main.cc:1186-1207
 * (rotation).  w_host (k) and q_host (k x k) may be NULL. */
ttg_status ttg_rayleigh_ritz(ttg_op* op, ttg_block* X, int32_t rotate, double* w_host,
                             double* q_host);

/* X <- X Q with Q k x k column-major on the host.  main.cc:1186-1207. */
ttg_status ttg_rotate(ttg_op* op, ttg_block* X, const double* q_host);

/* Lanczos spectral bounds with (H_loc + C^T D C).  Replaces
 * EigenSolver::computeUpperBoundWithLanczos (eigensolver/EigenSolver.h:40-44,
 * eigensolver/EigenSolver.cc:186-388): upper = |lambda_max(T)| + ||f||,
 * lower = lambda_min(T).  v0 (length n) is the start vector; the reference
 * draws it with VecSetRandom. */
ttg_status ttg_lanczos_bounds(ttg_op* op, const double* v0_host, int32_t max_iter,
                              double* upper, double* lower);

/* One ChFSI pass as main.cc:1047-1115 runs it: filter, Cholesky-QR,
 * Rayleigh-Ritz (eigenvalues to w_host, optional), and, if rotate != 0,
 * the rotation X <- X Q.  Where the reference's orth would meet a
 * non-positive pivot (the filter has driven columns of a wide block towards
 * the same eigenvectors), the pass does not fail: it orthonormalises with
 * shifted Cholesky-QR steps on the unit-diagonal Gram matrix (shift 1e-8)
 * followed by two plain ones, which keeps the column span and turns
 * dependent columns into fresh directions; ttg_op_info counts those steps
 * (shifted_orth). */
ttg_status ttg_chfsi_pass(ttg_op* op, ttg_block* X, int32_t m, double a, double b,
                          double a0, ttg_sched sched, int32_t rotate, double* w_host);

/* ---- operator values for a new potential (SCF) ----------------------------- */

/* 1-D stiffness (int psi' psi') and overlap matrices of the basis, r_d x r_d
 * row-major (dft/ProjectHamiltonianSparse.cc:577-676).  Needs an op created
 * with ttg_op_create_tucker. */
ttg_status ttg_op_set_kinetic(ttg_op* op, const double* dx, const double* dy, const double* dz,
                              const double* mx, const double* my, const double* mz);
/* Recompute the values of H_loc on its fixed pattern for an effective potential
 * in Tucker form, V = sum_abc G_abc u_a v_b w_c (G x-fastest, ranks pot_ranks):
 * H = 0.5 (DX MY MZ + MX DY MZ + MX MY DZ) + sum_abc G_abc PX_a (x) PY_b (x) PZ_c
 * with PX_a[i][j] = int psi_i u_a psi_j given as (ra x rx x rx) row-major
 * (Create_Hloc, dft/ProjectHamiltonianSparse.cc:330-575, on the device).
 * Entries the pattern does not hold are not created. */
ttg_status ttg_op_update_potential(ttg_op* op, const int32_t* pot_ranks, const double* G,
                                   const double* px, const double* py, const double* pz);
/* ttg_op_update_potential with G and the potential matrices in device memory,
 * on the op's stream, without synchronising. */
ttg_status ttg_op_update_potential_device(ttg_op* op, const int32_t* pot_ranks,
                                          const double* g_dev, const double* px_dev,
                                          const double* py_dev, const double* pz_dev);

/* ---- SCF grid kernels (FP64, device pointers, x-fastest fields) ------------ */

/* Sequentially truncated HOSVD (TuckerMPI::STHOSVD as used at main.cc:951-955
 * and tensor/TensorUtils.cc:245-264): per mode, the eigenvectors of the mode
 * Gram matrix, keeping the smallest rank whose discarded eigenvalues sum to
 * at most eps^2 ||T||^2 / 3 (capped by max_ranks when not NULL); eps 0
 * keeps exactly max_ranks (the fixed-rank form of main.cc:952-956).  Outputs:
 * ranks, core (x-fastest), factors u_d (n_d x r_d column-major) -- all device
 * buffers sized for the caps. */
ttg_status ttg_tucker_sthosvd(ttg_op* op, const double* t_dev, const int32_t* dims, double eps,
                              const int32_t* max_ranks, int32_t* ranks_out, double* core_dev,
                              double* u0_dev, double* u1_dev, double* u2_dev);
/* core x1 U0 x2 U1 x3 U2 onto an n0 x n1 x n2 grid (Tucker::ttm chain). */
ttg_status ttg_tucker_reconstruct(const double* core_dev, const int32_t* ranks,
                                  const double* u0_dev, const double* u1_dev,
                                  const double* u2_dev, const int32_t* dims, double* out_dev,
                                  void* stream);
/* LDA exchange-correlation potential (added to v when accumulate_v) and energy
 * density e = eps_xc(rho) rho (dft/KSDFTPotential.cc:127-267,
 * dft/KSDFTEnergyFunctional.cc:27-56).  v or e may be NULL. */
ttg_status ttg_grid_lda(const double* rho_dev, int64_t n, double* v_dev, double* e_dev,
                        int32_t accumulate_v, void* stream);
/* result = sum f g wx wy wz (g may be NULL): compute3DIntegral
 * (dft/KSDFTEnergyFunctional.cc:169-192) and the weighted inner products of
 * the Anderson mixing (dft/AndersonMixing.cc:150-265).  Fixed summation order. */
ttg_status ttg_grid_integrate(const double* f_dev, const double* g_dev, const int32_t* dims,
                              const double* wx_dev, const double* wy_dev, const double* wz_dev,
                              double* result, void* stream);
/* out[i,j,l] (+)= sum_a coef[a] fx[a,i] fy[a,j] fz[a,l]: superposition of
 * separable per-atom fields on a tensor grid -- the atomic-density initial
 * guess (InitialGuess::initializeRhoFromRadiusFile, dft/InitialGuess.cc:
 * 573-681) and the Gaussian-well local potential.  fx is (nterms x n0). */
ttg_status ttg_grid_cp_sum(int32_t nterms, const double* coef_dev, const double* fx_dev,
                           const double* fy_dev, const double* fz_dev, const int32_t* dims,
                           double* out_dev, int32_t accumulate, void* stream);
/* out -= sum_a z_a erf(|r - R_a| / width) / |r - R_a|: the exact electrostatic
 * potential of Gaussian ionic charges (pos: natoms x 3), which makes the
 * synthetic systems neutral under the Hartree term. */
ttg_status ttg_grid_ion_potential(int32_t natoms, const double* pos_dev, const double* z_dev,
                                  double width, const double* gx_dev, const double* gy_dev,
                                  const double* gz_dev, const int32_t* dims, double* out_dev,
                                  void* stream);
/* out = sum_m coef[m] fields[m] (|.| when take_abs), up to 24 fields
 * (dft/AndersonMixing.cc:267-316). */
ttg_status ttg_grid_lincomb(int32_t nterms, const double* const* fields_dev, const double* coef,
                            int64_t n, double* out_dev, int32_t take_abs, void* stream);

/* ---- Fermi level, density, Hartree --------------------------------------- */

/* Fermi level by Newton on sum_i 2 f_i = n_electrons and the occupations f_i.
 * Replaces KSDFTEnergyFunctional::computeFermiEnergy
 * (dft/KSDFTEnergyFunctional.cc:76-124) and the occupancy loop of
 * main.cc:1239-1272.  kT = kb*T in Ha.  Runs in FP64 on the GPU. */
ttg_status ttg_fermi(ttg_op* op, int32_t k, const double* eig_host, double n_electrons,
                     double kT, int32_t max_iter, double* mu, double* occ_host);

/* Nodal density rho(x,y,z) = sum_i 2 f_i (c_i x1 Ux x2 Uy x3 Uz)^2 where c_i
 * is column i of X (an rx*ry*rz Tucker core, x fastest) and Ux (nx x rx),
 * Uy, Uz (column-major) are the basis values at the nodes.  Output is
 * nx*ny*nz, x fastest, host memory.  Replaces the per-state reconstruction of
 * ProjectHamiltonianSparse::computeRhoOut (dft/ProjectHamiltonianSparse.cc:
 * 1021-1075).  Runs in chunks of states (the intermediates stay within a
 * fixed budget, 3 GiB unless TTG_DENSITY_CHUNK_BYTES says otherwise): three
 * persistent tcgen05 mode products of FP32 operands cut into exact integer
 * BF16 slices (see ttg_tc_gemm), the last one squaring, weighting and summing
 * over the chunk's states in double-FP32 inside its epilogue, so the
 * orbitals on the grid are never written to memory; rho is FP64. */
ttg_status ttg_density(ttg_op* op, const ttg_block* X, const double* occ_host,
                       int32_t rx, int32_t ry, int32_t rz,
                       int32_t nx, int32_t ny, int32_t nz,
                       const double* ux, const double* uy, const double* uz,
                       double* rho_host);
/* ttg_density on device data, on the op's stream, into the op's grow-only
 * work buffers (no host copy of rho, no synchronisation; a bounded-wait
 * timeout is reported by ttg_op_sync).  ranks = (rx, ry, rz), n = (nx, ny,
 * nz): host arrays; u*_dev: FP64 nodal basis values, n_d x r_d column-major;
 * rho_dev: FP64, nx*ny*nz, x fastest, overwritten (added to when
 * accumulate). */
ttg_status ttg_density_device(ttg_op* op, const ttg_block* X, const double* occ_host,
                              const int32_t* ranks, const int32_t* n, const double* ux_dev,
                              const double* uy_dev, const double* uz_dev, double* rho_dev,
                              int32_t accumulate);

/* Hartree potential by the Gaussian kernel expansion
 *   V(i,j,l) = sum_t w_t sum_abc G_abc Fx_t[i,a] Fy_t[j,b] Fz_t[l,c]
 *   Fx_t[i,a] = sum_q wq_q exp(-alpha_t (x_i - xq_q)^2) Ux[q,a]
 * (dft/KSDFTPotential.cc:269-340, factor integrals :440-599, per-term
 * contraction :601-658).  G is rx*ry*rz (x fastest); Ux is nqx x rx
 * column-major values of the density's Tucker factors at the quadrature
 * points xq with weights wq (J*w); the target grid is x (nx points).
 * alpha and omega are the already-scaled expansion coefficients.
 * The factor integrals run in FP64 on the CUDA cores (one launch per
 * direction); the three mode products are persistent tcgen05 launches of
 * FP32 operands cut into exact integer BF16 slices (see ttg_tc_gemm), the
 * last one summing the K terms in double-FP32, one group per term, so the
 * error is that of the FP32 operands whatever K.  Output nx*ny*nz, x
 * fastest, FP64, host memory.  kernel_ms: device time of the three
 * contractions.  Needs no op (creates its own stream); device memory is
 * released on return. */
ttg_status ttg_hartree(int32_t K, const double* alpha, const double* omega,
                       int32_t rx, int32_t ry, int32_t rz, const double* G,
                       int32_t nqx, int32_t nqy, int32_t nqz,
                       const double* xq, const double* yq, const double* zq,
                       const double* wqx, const double* wqy, const double* wqz,
                       const double* ux, const double* uy, const double* uz,
                       int32_t nx, int32_t ny, int32_t nz,
                       const double* x, const double* y, const double* z,
                       double* v_host, float* kernel_ms);

/* ttg_hartree on device data, on the op's stream, into the op's grow-only
 * work buffers (no allocation once they have grown, no host copy, no
 * synchronisation; a bounded-wait timeout is reported by ttg_op_sync).
 * alpha_dev, omega_dev: K values; ranks, nq, n: host arrays of 3; g_dev: the
 * core, x fastest; xq_dev[d], wq_dev[d]: nq[d] quadrature points and J*w
 * weights; u_dev[d]: nq[d] x ranks[d] column-major; x_dev[d]: n[d] target
 * points; v_dev: n0*n1*n2 FP64, x fastest.  Same replacement and arithmetic
 * as ttg_hartree. */
ttg_status ttg_hartree_device(ttg_op* op, int32_t K, const double* alpha_dev,
                              const double* omega_dev, const int32_t* ranks, const double* g_dev,
                              const int32_t* nq, const double* const* xq_dev,
                              const double* const* wq_dev, const double* const* u_dev,
                              const int32_t* n, const double* const* x_dev, double* v_dev);

/* C = A B^T on the tensor cores, FP32 operands, FP64 result: A (m x k) and B
 * (n x k) row-major with leading dimensions lda, ldb (multiples of 4, base
 * addresses 16-byte aligned), C (m x n) row-major with leading dimension ldc.
 * The K range is cut into `groups` groups of equal whole 16-value chunks (at
 * most 192 values each); each group's operands are cut into three integer
 * BF16 slices on a grid set by the group's largest |value|, their products
 * accumulate exactly in tensor memory (integer-valued operands come out
 * exact), and the groups are summed in double-FP32.  The contraction engine
 * of ttg_hartree and ttg_density, exposed for tests and as a library GEMM;
 * no counterpart in the reference.  Allocates a few bytes of scratch;
 * synchronises the stream. */
ttg_status ttg_tc_gemm(int64_t m, int64_t n, int64_t k, const float* a_dev, int64_t lda,
                       const float* b_dev, int64_t ldb, int32_t groups, double* c_dev,
                       int64_t ldc, void* stream);

/* Hartree energy of a Tucker density on its own quadrature grid,
 *   E_H = 1/2 sum_q sum_q' w_q rho_q K(q, q') w_q' rho_q'
 *       = 1/2 sum_t omega_t <G, G x1 Kx_t x2 Ky_t x3 Kz_t>,
 *   Kx_t = (Wx Ux)^T E_t (Wx Ux),  E_t[q, q'] = exp(-alpha_t (xq_q - xq_q')^2),
 * the quadrature of the term 1/2 int rho V_H(rho) of the total energy
 * (main.cc:1315-1401 with V_H from dft/KSDFTPotential.cc:269-340), from FP64
 * data without forming V_H on the grid: three double-FP32 GEMMs per term
 * (about 2^-47 relative per product) and FP64 dot products.  ranks = (rx, ry,
 * rz), G x fastest, nq[d] quadrature points xq_d with weights wq_d, U_d
 * nq[d] x r[d] column-major; all host memory.  Needs no op. */
ttg_status ttg_hartree_energy(int32_t K, const double* alpha, const double* omega,
                              const int32_t* ranks, const double* G, const int32_t* nq,
                              const double* xq, const double* yq, const double* zq,
                              const double* wqx, const double* wqy, const double* wqz,
                              const double* ux, const double* uy, const double* uz,
                              double* energy);

/* ---- learned initial density (no counterpart in the reference; its guess
 * is the superposition of atomic densities, dft/InitialGuess.cc:573-681,
 * which stays the fallback) --------------------------------------------- */

/* Pairwise Gaussian radial descriptors of each atom (pos: natoms x 3, bohr):
 *   out[a][m] = sum_{b != a} exp(-eta (r_ab - mu_m)^2) fc(r_ab),
 *   mu_m = mu0 + m dmu, fc(r) = (cos(pi r / rc) + 1) / 2 for r < rc.
 * out: natoms x n_features, host memory. */
ttg_status ttg_atom_descriptors(int32_t natoms, const double* pos, int32_t n_features, double mu0,
                                double dmu, double eta, double rc, float* out);

/* Multilayer perceptron, FP32: sizes[0..n_layers], tanh hidden layers, linear
 * output; parameters packed per layer as W (in x out, row-major) then b. */
typedef struct ttg_mlp ttg_mlp;
ttg_status ttg_mlp_create(int32_t n_layers, const int32_t* sizes, ttg_mlp** out);
void ttg_mlp_destroy(ttg_mlp* m);
int64_t ttg_mlp_num_params(const ttg_mlp* m);
/* Host FP32 parameter vectors; set also resets the optimiser state. */
ttg_status ttg_mlp_set_params(ttg_mlp* m, const float* p);
ttg_status ttg_mlp_get_params(ttg_mlp* m, float* p);
/* y (n x out) = network(x (n x in)), host arrays. */
ttg_status ttg_mlp_forward(ttg_mlp* m, const float* x, int32_t n, float* y);
/* Loss = mean over samples of sum_j (y_j - t_j)^2 and its gradient with
 * respect to the parameters (host arrays). */
ttg_status ttg_mlp_gradients(ttg_mlp* m, const float* x, const float* t, int32_t n, float* grad,
                             float* loss);
/* Minibatch Adam (decoupled weight decay on the weights) for `epochs` passes
 * over (x, t); samples reshuffled every epoch from `seed`; the mean loss of
 * each epoch into loss_per_epoch (may be NULL). */
ttg_status ttg_mlp_train(ttg_mlp* m, const float* x, const float* t, int32_t n, int32_t epochs,
                         int32_t batch, float lr, float weight_decay, uint64_t seed,
                         float* loss_per_epoch);

#ifdef __cplusplus
}
#endif

#endif /* TTG_H_ */
