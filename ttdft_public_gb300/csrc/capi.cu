// extern "C" entry points of libttg (declared in include/ttg.h).
//
// Host orchestration of the device kernels: operator and block lifetime,
// the Chebyshev recurrence scalars (eigensolver/ChebyShevFilter.cc:68-75,
// :129-134), Cholesky-QR, Rayleigh-Ritz and Lanczos.  Every launch goes to the
// op's own stream; nothing here computes on the CPU.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "ttg_internal.cuh"

using namespace ttg;

namespace {

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

ttg_status ensure(DevBuf& b, size_t bytes, ttg_op* op) {
  if (b.bytes >= bytes) return TTG_OK;
  const size_t old = b.bytes;
  TTG_TRY(b.alloc(bytes));
  op->device_bytes += (int64_t)bytes - (int64_t)old;
  return TTG_OK;
}

size_t block_bytes(const ttg_op* op, size_t elem) {
  return (size_t)(op->n + op->nproj) * (size_t)op->ld * elem;
}

ttg_status read_status(ttg_op* op, int* host_status) {
  TTG_CUDA_TRY(cudaMemcpyAsync(host_status, op->status.p, sizeof(int), cudaMemcpyDeviceToHost,
                               op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  return TTG_OK;
}

ttg_status check_block(const ttg_op* op, const ttg_block* b) {
  if (!op || !b || b->op != op) return TTG_BAD_ARG;
  return TTG_OK;
}

// S = X^T Y (k x k, column-major) from FP64 blocks: on the tensor cores
// (ozgemm.cu) where the operands allow, else the double-FP32 CUDA-core kernel.
ttg_status gram_fp64(ttg_op* op, const double* X, const double* Y, int k, double* S, bool sym) {
  const OzOperand A{X, k, op->n, op->ld, true}, B{Y, k, op->n, op->ld, true};
  if (ozgemm_supported(A, B)) return ozgemm(op, A, B, S, 1, k, sym);
  return gram_tn(op, X, Y, k, S, sym);
}

// out = X Q (transQ = 0) or X Q^T (transQ = 1; lower: Q lower triangular),
// Q column-major k x k; the same choice of kernel as gram_fp64.  kscale: Q
// undoes the columns' scales of X (Q = L^-1 of X's Cholesky-QR); the
// product then runs on K scales taken from X's columns.
ttg_status product_fp64(ttg_op* op, const double* X, const double* Q, double* out, int k,
                        int transQ, bool lower, bool kscale = false) {
  // B(n = q, k = p) = Qop[p, q]: Q[p + q k] (K-major) or, transposed, Q[q + p k] (MN-major)
  const OzOperand A{X, op->n, k, op->ld, false}, B{Q, k, k, k, transQ != 0};
  const OzOperand cols{X, k, op->n, op->ld, true};
  if (ozgemm_supported(A, B))
    return ozgemm(op, A, B, out, op->ld, 1, false, transQ && lower, kscale ? &cols : nullptr);
  return gemm_nn_small(op, X, Q, out, k, transQ, lower);
}

}  // namespace

namespace ttg {
std::atomic<long long> g_kernel_launches{0};
}

namespace ttg {

static ttg_status kt_flush(ttg_op* op) {
  KernelTimer& T = op->kt;
  if (T.used == 0) return TTG_OK;
  TTG_CUDA_TRY(cudaEventSynchronize(T.ev[2 * T.used - 1]));
  for (int i = 0; i < T.used; ++i) {
    float ms = 0.f;
    TTG_CUDA_TRY(cudaEventElapsedTime(&ms, T.ev[2 * i], T.ev[2 * i + 1]));
    T.ms[T.kind[i]] += ms;
    T.count[T.kind[i]]++;
  }
  T.used = 0;
  return TTG_OK;
}

ttg_status kt_begin(ttg_op* op, int kind) {
  KernelTimer& T = op->kt;
  if (!T.on) return TTG_OK;
  if (T.used == KernelTimer::kPairs) TTG_TRY(kt_flush(op));
  T.kind[T.used] = kind;
  TTG_CUDA_TRY(cudaEventRecord(T.ev[2 * T.used], op->stream));
  return TTG_OK;
}

ttg_status kt_end(ttg_op* op) {
  KernelTimer& T = op->kt;
  if (!T.on) return TTG_OK;
  TTG_CUDA_TRY(cudaEventRecord(T.ev[2 * T.used + 1], op->stream));
  T.used++;
  return TTG_OK;
}

}  // namespace ttg

extern "C" {

const char* ttg_version(void) { return "ttg 0.1 (sm_103a)"; }

int64_t ttg_kernel_launches(void) {
  return (int64_t)ttg::g_kernel_launches.load(std::memory_order_relaxed);
}

const char* ttg_status_string(ttg_status s) {
  switch (s) {
    case TTG_OK: return "ok";
    case TTG_BAD_ARG: return "bad argument";
    case TTG_BAD_CSR: return "malformed CSR";
    case TTG_OOM: return "out of device memory";
    case TTG_NOT_SPD: return "matrix not positive definite";
    case TTG_NONFINITE: return "non-finite value";
    case TTG_TIMEOUT: return "device wait timed out";
    case TTG_CUDA_ERR: return "CUDA error";
    case TTG_NO_DEVICE: return "no sm_100+ device";
    case TTG_NOT_CONVERGED: return "iteration did not converge";
  }
  return "unknown";
}

ttg_status ttg_device_query(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor) {
  int dev = 0, n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return TTG_NO_DEVICE;
  }
  TTG_CUDA_TRY(cudaGetDevice(&dev));
  cudaDeviceProp p;
  TTG_CUDA_TRY(cudaGetDeviceProperties(&p, dev));
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  return p.major >= 10 ? TTG_OK : TTG_NO_DEVICE;
}

ttg_status ttg_op_create(int64_t n, const int64_t* h_row_ptr, const int32_t* h_col,
                         const double* h_val, int32_t nproj, const int64_t* c_row_ptr,
                         const int32_t* c_col, const double* c_val, const double* d,
                         int32_t max_k, ttg_op** out) {
  return ttg_op_create_tucker(n, h_row_ptr, h_col, h_val, nproj, c_row_ptr, c_col, c_val, d,
                              nullptr, max_k, out);
}

ttg_status ttg_op_create_tucker(int64_t n, const int64_t* h_row_ptr, const int32_t* h_col,
                                const double* h_val, int32_t nproj, const int64_t* c_row_ptr,
                                const int32_t* c_col, const double* c_val, const double* d,
                                const int32_t* tucker_ranks, int32_t max_k, ttg_op** out) {
  if (!out || n <= 0 || n > INT32_MAX - 65536 || nproj < 0 || nproj > 65536 || max_k <= 0 ||
      max_k > 4096 || !h_row_ptr)
    return TTG_BAD_ARG;
  if (tucker_ranks && (int64_t)tucker_ranks[0] * tucker_ranks[1] * tucker_ranks[2] != n)
    return TTG_BAD_ARG;
  *out = nullptr;
  int32_t smc, ma, mi;
  TTG_TRY(ttg_device_query(&smc, &ma, &mi));
  ttg_op* op = new ttg_op();
  cudaGetDevice(&op->device);
  op->n = n;
  op->nproj = nproj;
  op->max_k = max_k;
  op->ld = round_up(max_k, 8);
  op->keep_pattern = tucker_ranks != nullptr;
  if (tucker_ranks)
    for (int d = 0; d < 3; ++d) op->pattern.r[d] = tucker_ranks[d];
  auto fail = [&](ttg_status s) {
    ttg_op_destroy(op);
    return s;
  };
  if (cudaStreamCreateWithFlags(&op->stream, cudaStreamDefault) != cudaSuccess)
    return fail(TTG_CUDA_ERR);
  for (int i = 0; i < kMaxSlots; ++i)
    if (cudaEventCreate(&op->ev[i]) != cudaSuccess) return fail(TTG_CUDA_ERR);
  ttg_status s = build_row_groups(op, n, h_row_ptr, h_col, h_val, nproj, c_row_ptr, c_col,
                                  c_val, d);
  if (s != TTG_OK) return fail(s);
  const char* dis = getenv("TTG_DISABLE_TC");
  op->tc_disabled = dis && dis[0] == '1';
  if (!op->tc_disabled) {
    // the mma.sync tiles serve block widths that are not multiples of 16;
    // an op for wide blocks of multiples of 16 (the tcgen05 degrees run them
    // in column blocks) does without them and their memory
    if (!(max_k > 256 && max_k % 16 == 0)) {
      s = build_tiles(op, n, h_row_ptr, h_col, h_val, nproj, c_row_ptr, c_col, c_val,
                      tucker_ranks);
      if (s != TTG_OK) return fail(s);
    }
    s = build_umma_tiles(op, n, h_row_ptr, h_col, h_val, nproj, c_row_ptr, c_col, c_val,
                         tucker_ranks);
    if (s != TTG_OK) return fail(s);
  }
  const int64_t kmax = std::max<int64_t>(max_k, kMaxLanczos);
  if ((s = ensure(op->kk0, kmax * kmax * 8, op)) != TTG_OK) return fail(s);
  if ((s = ensure(op->kk1, kmax * kmax * 8, op)) != TTG_OK) return fail(s);
  if ((s = ensure(op->kk2, kmax * kmax * 8, op)) != TTG_OK) return fail(s);
  if ((s = ensure(op->kk3, (kmax * kmax + 6 * kmax + 64) * 8, op)) != TTG_OK) return fail(s);
  if ((s = ensure(op->scal, (kScalJacobi + 4 * (kmax + 2) + kmax) * 8, op)) != TTG_OK)
    return fail(s);
  if ((s = ensure(op->status, 64, op)) != TTG_OK) return fail(s);
  if ((s = ensure(op->w64, block_bytes(op, 8), op)) != TTG_OK) return fail(s);
  if (cudaMemsetAsync(op->status.p, 0, 64, op->stream) != cudaSuccess) return fail(TTG_CUDA_ERR);
  if (cudaStreamSynchronize(op->stream) != cudaSuccess) return fail(TTG_CUDA_ERR);
  *out = op;
  return TTG_OK;
}

ttg_status ttg_op_destroy(ttg_op* op) {
  if (!op) return TTG_BAD_ARG;
  if (op->stream) cudaStreamSynchronize(op->stream);
  DevBuf* bufs[] = {&op->rg.gptr, &op->rg.gcol, &op->rg.v64, &op->rg.v32, &op->rg.v16,
                    &op->rg.vdf,  &op->wdf,     &op->wpart,
                    &op->C.ptr,   &op->C.col,   &op->C.val,  &op->C.val32, &op->w32a,
                    &op->w32b,    &op->w16a,    &op->w16b,   &op->w64,     &op->kk0,
                    &op->kk1,     &op->kk2,     &op->kk3,     &op->eigbuf,  &op->eigf,    &op->partial, &op->scal,   &op->status,
                    &op->tiles.tptr, &op->tiles.tcol, &op->tiles.rowmap, &op->tiles.v32,
                    &op->tiles.v16, &op->pattern.row_ptr, &op->pattern.col,
                    &op->pattern.rg_pos, &op->pattern.tile_base, &op->pattern.tile_slot,
                    &op->pattern.umma_pos, &op->pattern.umma_row,
                    &op->pattern.kin, &op->pattern.work, &op->pattern.work2};
  for (DevBuf* b : bufs) b->release();
  for (int i = 0; i < kMaxSlots; ++i)
    if (op->ev[i]) cudaEventDestroy(op->ev[i]);
  for (cudaEvent_t e : op->kt.ev)
    if (e) cudaEventDestroy(e);
  if (op->stream) cudaStreamDestroy(op->stream);
  delete op;
  return TTG_OK;
}

ttg_status ttg_op_kernel_timing(ttg_op* op, int32_t enable) {
  if (!op) return TTG_BAD_ARG;
  KernelTimer& T = op->kt;
  if (enable && !T.on) {
    if (T.ev.empty()) {
      T.ev.resize(2 * KernelTimer::kPairs, nullptr);
      T.kind.resize(KernelTimer::kPairs, 0);
      for (cudaEvent_t& e : T.ev) TTG_CUDA_TRY(cudaEventCreate(&e));
    }
    T.on = true;
  } else if (!enable) {
    if (T.on) TTG_TRY(kt_flush(op));
    T.on = false;
    for (int i = 0; i < TTG_KT_KINDS; ++i) {
      T.ms[i] = 0.0;
      T.count[i] = 0;
    }
  }
  return TTG_OK;
}

ttg_status ttg_op_kernel_time(ttg_op* op, int32_t kind, double* ms_total, int64_t* launches) {
  if (!op || kind < 0 || kind >= TTG_KT_KINDS || !ms_total || !launches) return TTG_BAD_ARG;
  TTG_TRY(kt_flush(op));
  *ms_total = op->kt.ms[kind];
  *launches = op->kt.count[kind];
  return TTG_OK;
}

ttg_status ttg_op_info(const ttg_op* op, ttg_op_info_t* info) {
  if (!op || !info) return TTG_BAD_ARG;
  info->n = op->n;
  info->nnz_h = op->nnz_h;
  info->nnz_c = op->nnz_c;
  info->nproj = op->nproj;
  info->group_rows = kGroupRows;
  info->n_groups = op->rg.n_groups;
  info->stored_cols = op->rg.slots;
  info->fill = op->rg.slots > 0
                   ? (double)(op->nnz_h + op->nnz_c) / ((double)kGroupRows * op->rg.slots)
                   : 0.0;
  info->device_bytes = op->device_bytes;
  info->launches = op->launches;
  info->n_tiles = op->tiles.n_tiles;
  info->tile_slots = op->tiles.slots;
  info->tile_fill = op->tiles.slots > 0
                        ? (double)(op->nnz_h + op->nnz_c) / (64.0 * op->tiles.slots)
                        : 0.0;
  info->umma_tiles = op->umma.n_tiles;
  info->shifted_orth = op->shifted_orth;
  info->umma_slots = op->umma.slots;
  return TTG_OK;
}

void* ttg_op_stream(ttg_op* op) { return op ? (void*)op->stream : nullptr; }

ttg_status ttg_op_set_rr_precision(ttg_op* op, int32_t prec) {
  if (!op || (prec != TTG_PREC_FP64 && prec != TTG_PREC_DF64)) return TTG_BAD_ARG;
  op->rr_prec = prec;
  return TTG_OK;
}

ttg_status ttg_op_sync(ttg_op* op) {
  if (!op) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  TTG_TRY(umma_check_error(op));
  return hartree_error(op);
}

ttg_status ttg_op_record(ttg_op* op, int32_t slot) {
  if (!op || slot < 0 || slot >= kMaxSlots) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaEventRecord(op->ev[slot], op->stream));
  return TTG_OK;
}

ttg_status ttg_op_elapsed_ms(ttg_op* op, int32_t s0, int32_t s1, float* ms) {
  if (!op || !ms || s0 < 0 || s1 < 0 || s0 >= kMaxSlots || s1 >= kMaxSlots) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaEventSynchronize(op->ev[s1]));
  TTG_CUDA_TRY(cudaEventElapsedTime(ms, op->ev[s0], op->ev[s1]));
  return TTG_OK;
}

// ------------------------------------------------------------- blocks ----

ttg_status ttg_block_create(ttg_op* op, int32_t k, ttg_block** out) {
  if (!op || !out || k <= 0 || k > op->max_k) return TTG_BAD_ARG;
  ttg_block* b = new ttg_block();
  b->op = op;
  b->k = k;
  ttg_status s = b->x.alloc(block_bytes(op, 8));
  if (s != TTG_OK) {
    delete b;
    return s;
  }
  cudaMemsetAsync(b->x.p, 0, b->x.bytes, op->stream);
  *out = b;
  return TTG_OK;
}

ttg_status ttg_block_destroy(ttg_block* b) {
  if (!b) return TTG_BAD_ARG;
  // cudaFree waits for the device; the op may already be gone, so it is not
  // touched here.
  b->x.release();
  delete b;
  return TTG_OK;
}

int32_t ttg_block_cols(const ttg_block* b) { return b ? b->k : 0; }

ttg_status ttg_block_set(ttg_block* b, const double* x, int64_t ld) {
  if (!b || !x || ld < b->op->n) return TTG_BAD_ARG;
  ttg_op* op = b->op;
  const int64_t n = op->n;
  for (int j = 0; j < b->k; ++j)
    for (int64_t i = 0; i < n; ++i)
      if (!std::isfinite(x[i + j * ld])) return TTG_NONFINITE;
  // stage column-major in w64, then transpose into the row-major block
  TTG_CUDA_TRY(cudaMemcpy2DAsync(op->w64.p, n * 8, x, ld * 8, n * 8, b->k,
                                 cudaMemcpyHostToDevice, op->stream));
  TTG_TRY(colmajor_to_rows(op, op->w64.as<double>(), n, b->x.as<double>(), op->ld, n, b->k));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  return TTG_OK;
}

ttg_status ttg_block_get(ttg_block* b, double* x, int64_t ld) {
  if (!b || !x || ld < b->op->n) return TTG_BAD_ARG;
  ttg_op* op = b->op;
  const int64_t n = op->n;
  TTG_TRY(rows_to_colmajor(op, b->x.as<double>(), op->ld, op->w64.as<double>(), n, n, b->k));
  TTG_CUDA_TRY(cudaMemcpy2DAsync(x, ld * 8, op->w64.p, n * 8, n * 8, b->k,
                                 cudaMemcpyDeviceToHost, op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  return TTG_OK;
}

ttg_status ttg_block_set_device(ttg_block* b, const double* x, int64_t ld) {
  if (!b || !x || ld < b->op->n) return TTG_BAD_ARG;
  return colmajor_to_rows(b->op, x, ld, b->x.as<double>(), b->op->ld, b->op->n, b->k);
}

ttg_status ttg_block_get_device(ttg_block* b, double* x, int64_t ld) {
  if (!b || !x || ld < b->op->n) return TTG_BAD_ARG;
  return rows_to_colmajor(b->op, b->x.as<double>(), b->op->ld, x, ld, b->op->n, b->k);
}

ttg_status ttg_block_copy(ttg_block* dst, const ttg_block* src) {
  if (!dst || !src || dst->op != src->op || dst->k != src->k) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaMemcpyAsync(dst->x.p, src->x.p, (size_t)dst->op->n * dst->op->ld * 8,
                               cudaMemcpyDeviceToDevice, dst->op->stream));
  return TTG_OK;
}

// ------------------------------------------------------------ hot path ----

ttg_status ttg_cheb_filter(ttg_op* op, ttg_block* X, int32_t m, double a, double b, double a0,
                           ttg_sched sched) {
  TTG_TRY(check_block(op, X));
  if (m < 0 || !(b > a) || !std::isfinite(a) || !std::isfinite(b) || !std::isfinite(a0))
    return TTG_BAD_ARG;
  auto okp = [](int p) { return p == TTG_PREC_FP64 || p == TTG_PREC_FP32 || p == TTG_PREC_BF16; };
  if (!okp(sched.low) || !okp(sched.high) || sched.n_low < 0) return TTG_BAD_ARG;
  const int k = X->k;
  const int steps = sched.return_prev ? m - 1 : m;
  if (steps <= 0) return TTG_OK;
  // recurrence scalars, eigensolver/ChebyShevFilter.cc:68-75 and :129-134
  const double e = (b - a) / 2.0, c = (b + a) / 2.0;
  double sigma = e / (a0 - c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  if (!std::isfinite(sigma)) return TTG_BAD_ARG;
  auto prec_of = [&](int d) { return d <= sched.n_low ? sched.low : sched.high; };
  auto bufs_for = [&](int p, void** x, void** y) -> ttg_status {
    if (p == TTG_PREC_FP64) {
      *x = X->x.p;
      *y = op->w64.p;
    } else if (p == TTG_PREC_FP32) {
      TTG_TRY(ensure(op->w32a, block_bytes(op, 4), op));
      TTG_TRY(ensure(op->w32b, block_bytes(op, 4), op));
      *x = op->w32a.p;
      *y = op->w32b.p;
    } else {
      TTG_TRY(ensure(op->w16a, block_bytes(op, 2), op));
      TTG_TRY(ensure(op->w16b, block_bytes(op, 2), op));
      *x = op->w16a.p;
      *y = op->w16b.p;
    }
    return TTG_OK;
  };
  int cur = prec_of(1);
  void *xb, *yb;
  TTG_TRY(bufs_for(cur, &xb, &yb));
  if (cur != TTG_PREC_FP64) TTG_TRY(launch_convert(op, TTG_PREC_FP64, cur, X->x.p, xb, op->n, k));
  // degree 1: Y = (sigma1/e) (H X - c X)
  double alpha = sigma1 / e, beta = -c * alpha;
  TTG_TRY(launch_proj_w(op, cur, xb, k));
  TTG_TRY(launch_cheb_step(op, cur, xb, nullptr, yb, k, alpha, beta, 0.0));
  for (int d = 2; d <= steps; ++d) {
    const int p = prec_of(d);
    if (p != cur) {
      void *nx, *ny;
      TTG_TRY(bufs_for(p, &nx, &ny));
      if (cur == TTG_PREC_FP64) {
        // FP64 buffers are X itself and w64: convert both down
        TTG_TRY(launch_convert(op, TTG_PREC_FP64, p, xb, nx, op->n, k));
        TTG_TRY(launch_convert(op, TTG_PREC_FP64, p, yb, ny, op->n, k));
      } else if (p == TTG_PREC_FP64) {
        TTG_TRY(launch_convert(op, cur, TTG_PREC_FP64, xb, op->w64.p, op->n, k));
        std::swap(op->w64.p, X->x.p);  // w64 now holds old X storage; fill Y next
        TTG_TRY(launch_convert(op, cur, TTG_PREC_FP64, yb, op->w64.p, op->n, k));
        nx = X->x.p;
        ny = op->w64.p;
      } else {
        TTG_TRY(launch_convert(op, cur, p, xb, nx, op->n, k));
        TTG_TRY(launch_convert(op, cur, p, yb, ny, op->n, k));
      }
      xb = nx;
      yb = ny;
      cur = p;
    }
    // Ynew = (2 sigma2/e)(H Y - c Y) - sigma sigma2 X, written over X
    const double sigma2 = 1.0 / (gamma - sigma);
    alpha = 2.0 * sigma2 / e;
    beta = -c * alpha;
    const double delta = -sigma * sigma2;
    TTG_TRY(launch_proj_w(op, cur, yb, k));
    TTG_TRY(launch_cheb_step(op, cur, yb, xb, xb, k, alpha, beta, delta));
    std::swap(xb, yb);
    sigma = sigma2;
  }
  // result is in yb
  if (cur == TTG_PREC_FP64) {
    if (yb != X->x.p) {
      // yb is w64: swap the storage so that X owns the result
      std::swap(op->w64.p, X->x.p);
    }
  } else {
    TTG_TRY(launch_convert(op, cur, TTG_PREC_FP64, yb, X->x.p, op->n, k));
  }
  return TTG_OK;
}

ttg_status ttg_apply_h(ttg_op* op, const ttg_block* X, ttg_block* HX) {
  TTG_TRY(check_block(op, X));
  TTG_TRY(check_block(op, HX));
  if (X->k != HX->k || X == HX) return TTG_BAD_ARG;
  ttg_block* Xm = const_cast<ttg_block*>(X);   // its projector rows are scratch
  TTG_TRY(launch_proj_w(op, TTG_PREC_FP64, Xm->x.p, X->k));
  TTG_TRY(launch_cheb_step(op, TTG_PREC_FP64, Xm->x.p, nullptr, HX->x.p, X->k, 1.0, 0.0, 0.0));
  return TTG_OK;
}

ttg_status ttg_gram(ttg_op* op, const ttg_block* X, const ttg_block* Y, double* s_host) {
  TTG_TRY(check_block(op, X));
  TTG_TRY(check_block(op, Y));
  if (X->k != Y->k) return TTG_BAD_ARG;
  const int k = X->k;
  TTG_TRY(gram_fp64(op, X->x.as<double>(), Y->x.as<double>(), k, op->kk0.as<double>(), false));
  if (s_host) {
    TTG_CUDA_TRY(cudaMemcpyAsync(s_host, op->kk0.p, (size_t)k * k * 8, cudaMemcpyDeviceToHost,
                                 op->stream));
    TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  }
  return TTG_OK;
}

namespace {

// One Cholesky-QR step.  shifted: factor D^-1 S D^-1 + 1e-8 I instead of S
// (D = sqrt(diag S)), which is positive definite whatever the columns' norms
// and their dependence, and apply X <- X (L^-1 D^-1)^T.  The column span is
// kept; a singular value sigma of the unit-scaled block becomes
// sigma / sqrt(sigma^2 + 1e-8): about 1 for sigma >> 1e-4 and sigma * 1e4
// below, so each shifted step divides a condition number above 1e4 by about
// 1e4 (shifted Cholesky-QR: Fukaya, Kannan, Nakatsukasa, Yamamoto and
// Yanagisawa, SIAM J. Sci. Comput. 42 (2020) A477-A503).
ttg_status chol_qr_step(ttg_op* op, ttg_block* X, bool shifted) {
  const int k = X->k;
  double* S = op->kk0.as<double>();
  double* L = op->kk1.as<double>();
  double* d = op->kk2.as<double>();
  TTG_TRY(kt_begin(op, TTG_KT_ORTH_GRAM));
  TTG_TRY(gram_fp64(op, X->x.as<double>(), X->x.as<double>(), k, S, true));
  TTG_TRY(kt_end(op));
  if (shifted) {
    int* bad = op->status.as<int>() + 1;
    TTG_TRY(unit_scale_shift(op, S, d, k, 1e-8, bad));
    int nbad = 0;
    TTG_CUDA_TRY(cudaMemcpyAsync(&nbad, bad, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
    TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
    if (nbad) {
      fprintf(stderr, "ttg: Cholesky-QR: %d of %d columns have a zero or non-finite norm\n",
              nbad, k);
      return TTG_NONFINITE;
    }
  }
  TTG_TRY(kt_begin(op, TTG_KT_ORTH_CHOL));
  TTG_TRY(cholesky_inv(op, S, L, k, op->status.as<int>()));
  TTG_TRY(kt_end(op));
  int st = 0;
  TTG_TRY(read_status(op, &st));
  if (st != 0) {
    if (shifted)
      fprintf(stderr, "ttg: shifted Cholesky-QR: pivot %d of %d not positive\n", st, k);
    return TTG_NOT_SPD;
  }
  if (shifted) TTG_TRY(scale_cols(op, L, d, k));
  TTG_TRY(kt_begin(op, TTG_KT_ORTH_UPDATE));
  // L^-T undoes the columns' scales of X: K scales from those columns keep
  // a column 1e-6 of the largest at full precision in the digit slicing
  TTG_TRY(product_fp64(op, X->x.as<double>(), L, op->w64.as<double>(), k, 1, true, true));
  TTG_TRY(kt_end(op));
  std::swap(op->w64.p, X->x.p);
  return TTG_OK;
}

// Orthonormalisation of a filtered block that must not fail: Cholesky-QR,
// and when its Gram matrix is not numerically positive definite (a block
// whose columns the filter has driven towards the same few eigenvectors),
// shifted steps until a plain Cholesky-QR succeeds, then one more plain step
// for orthogonality (shifted Cholesky-QR3).  A block with exactly dependent
// columns comes out with those directions replaced by rounding-level ones,
// orthonormal to the rest: the next filter pass treats them as new start
// vectors.
ttg_status chol_qr_robust(ttg_op* op, ttg_block* X, int* shifted_steps) {
  *shifted_steps = 0;
  ttg_status s = chol_qr_step(op, X, false);
  if (s == TTG_NOT_SPD && sync_launches())
    fprintf(stderr, "ttg: Cholesky-QR of the filtered block: non-positive pivot; shifted steps\n");
  for (int i = 0; s == TTG_NOT_SPD && i < 4; ++i) {
    TTG_TRY(chol_qr_step(op, X, true));
    ++*shifted_steps;
    s = chol_qr_step(op, X, false);
    if (s == TTG_OK) s = chol_qr_step(op, X, false);
  }
  return s;
}

}  // namespace

ttg_status ttg_chol_qr(ttg_op* op, ttg_block* X) {
  TTG_TRY(check_block(op, X));
  return chol_qr_step(op, X, false);
}

static ttg_status eig_device(ttg_op* op, int k, double* A, double* V, double* w_dev) {
  TTG_TRY(syev_device(op, A, V, w_dev, k, op->status.as<int>()));
  int st = 0;
  TTG_TRY(read_status(op, &st));
  return st == 0 ? TTG_OK : TTG_NOT_CONVERGED;
}

ttg_status ttg_syev(ttg_op* op, int32_t k, const double* a_host, double* w_host, double* v_host) {
  if (!op || k <= 0 || !a_host || (int64_t)k * k * 8 > (int64_t)op->kk0.bytes ||
      k > 4096)
    return TTG_BAD_ARG;
  for (int64_t i = 0; i < (int64_t)k * k; ++i)
    if (!std::isfinite(a_host[i])) return TTG_NONFINITE;
  TTG_CUDA_TRY(cudaMemcpyAsync(op->kk0.p, a_host, (size_t)k * k * 8, cudaMemcpyHostToDevice,
                               op->stream));
  double* wdev = op->scal.as<double>() + kScalEig;
  ttg_status s = eig_device(op, k, op->kk0.as<double>(), op->kk1.as<double>(), wdev);
  if (s != TTG_OK) return s;
  if (w_host)
    TTG_CUDA_TRY(cudaMemcpyAsync(w_host, wdev, (size_t)k * 8, cudaMemcpyDeviceToHost, op->stream));
  if (v_host)
    TTG_CUDA_TRY(cudaMemcpyAsync(v_host, op->kk1.p, (size_t)k * k * 8, cudaMemcpyDeviceToHost,
                                 op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  return TTG_OK;
}

ttg_status ttg_rayleigh_ritz(ttg_op* op, ttg_block* X, int32_t rotate, double* w_host,
                             double* q_host) {
  TTG_TRY(check_block(op, X));
  const int k = X->k;
  // HX into w64 (FP64 values), then P = X^T HX
  TTG_TRY(kt_begin(op, TTG_KT_RR_HX));
  TTG_TRY(launch_proj_w(op, TTG_PREC_FP64, X->x.p, k));
  if (op->rr_prec == TTG_PREC_DF64)
    TTG_TRY(launch_apply_df64(op, X->x.as<double>(), op->w64.as<double>(), k));
  else
    TTG_TRY(launch_cheb_step(op, TTG_PREC_FP64, X->x.p, nullptr, op->w64.p, k, 1.0, 0.0, 0.0));
  TTG_TRY(kt_end(op));
  TTG_TRY(kt_begin(op, TTG_KT_RR_GRAM));
  TTG_TRY(gram_fp64(op, X->x.as<double>(), op->w64.as<double>(), k, op->kk0.as<double>(), true));
  TTG_TRY(kt_end(op));
  double* wdev = op->scal.as<double>() + kScalEig;
  TTG_TRY(kt_begin(op, TTG_KT_RR_EIG));
  TTG_TRY(eig_device(op, k, op->kk0.as<double>(), op->kk1.as<double>(), wdev));
  TTG_TRY(kt_end(op));
  if (rotate) {
    TTG_TRY(kt_begin(op, TTG_KT_RR_ROTATE));
    TTG_TRY(product_fp64(op, X->x.as<double>(), op->kk1.as<double>(), op->w64.as<double>(), k, 0,
                         false));
    TTG_TRY(kt_end(op));
    std::swap(op->w64.p, X->x.p);
  }
  if (w_host)
    TTG_CUDA_TRY(cudaMemcpyAsync(w_host, wdev, (size_t)k * 8, cudaMemcpyDeviceToHost, op->stream));
  if (q_host)
    TTG_CUDA_TRY(cudaMemcpyAsync(q_host, op->kk1.p, (size_t)k * k * 8, cudaMemcpyDeviceToHost,
                                 op->stream));
  if (w_host || q_host) TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  return TTG_OK;
}

ttg_status ttg_rotate(ttg_op* op, ttg_block* X, const double* q_host) {
  TTG_TRY(check_block(op, X));
  if (!q_host) return TTG_BAD_ARG;
  const int k = X->k;
  TTG_CUDA_TRY(cudaMemcpyAsync(op->kk1.p, q_host, (size_t)k * k * 8, cudaMemcpyHostToDevice,
                               op->stream));
  TTG_TRY(product_fp64(op, X->x.as<double>(), op->kk1.as<double>(), op->w64.as<double>(), k, 0,
                       false));
  std::swap(op->w64.p, X->x.p);
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  TTG_TRY(ozgemm_error(op));
  return TTG_OK;
}

ttg_status ttg_lanczos_bounds(ttg_op* op, const double* v0_host, int32_t max_iter,
                              double* upper, double* lower) {
  if (!op || !v0_host || !upper || !lower || max_iter < 2 || max_iter > kMaxLanczos)
    return TTG_BAD_ARG;
  const int64_t n = op->n;
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v0_host[i])) return TTG_NONFINITE;
  // v, v_prev, H v as columns 0, 1, 2 of the FP64 scratch block
  double* base = op->w64.as<double>();
  double* v = base;
  double* vp = base + 1;
  double* hv = base + 2;
  if (op->ld < 3) return TTG_BAD_ARG;
  TTG_CUDA_TRY(cudaMemsetAsync(op->w64.p, 0, op->w64.bytes, op->stream));
  TTG_CUDA_TRY(cudaMemcpy2DAsync(v, op->ld * 8, v0_host, 8, 8, n, cudaMemcpyHostToDevice,
                                 op->stream));
  TTG_TRY(normalize(op, v));
  double* ab = op->scal.as<double>() + kScalLanczos;
  for (int it = 0; it < max_iter; ++it) {
    TTG_TRY(launch_proj_w(op, TTG_PREC_FP64, v, 1));
    TTG_TRY(launch_cheb_step(op, TTG_PREC_FP64, v, nullptr, hv, 1, 1.0, 0.0, 0.0));
    TTG_TRY(lanczos_step(op, v, vp, hv, ab, it));
  }
  std::vector<double> abh(2 * max_iter);
  TTG_CUDA_TRY(cudaMemcpyAsync(abh.data(), ab, abh.size() * 8, cudaMemcpyDeviceToHost, op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  // tridiagonal T (EigenSolver.cc:256-315): diag alpha_i, off-diag beta_{i-1}
  const int m = max_iter;
  std::vector<double> T((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) {
    T[i + (size_t)i * m] = abh[2 * i];
    if (i > 0) {
      T[i + (size_t)(i - 1) * m] = abh[2 * (i - 1) + 1];
      T[(i - 1) + (size_t)i * m] = abh[2 * (i - 1) + 1];
    }
  }
  const double f_norm = abh[2 * (m - 1) + 1];
  std::vector<double> w(m);
  TTG_TRY(ttg_syev(op, m, T.data(), w.data(), nullptr));
  *lower = w[0];
  *upper = f_norm + std::fabs(w[m - 1]);   // EigenSolver.cc:365-367
  return TTG_OK;
}

ttg_status ttg_chfsi_pass(ttg_op* op, ttg_block* X, int32_t m, double a, double b, double a0,
                          ttg_sched sched, int32_t rotate, double* w_host) {
  TTG_TRY(ttg_cheb_filter(op, X, m, a, b, a0, sched));
  TTG_TRY(umma_check_error(op));
  int shifted = 0;
  TTG_TRY(chol_qr_robust(op, X, &shifted));
  op->shifted_orth += shifted;
  TTG_TRY(ttg_rayleigh_ritz(op, X, rotate, w_host, nullptr));
  return ozgemm_error(op);
}

ttg_status ttg_fermi(ttg_op* op, int32_t k, const double* eig_host, double n_electrons, double kT,
                     int32_t max_iter, double* mu, double* occ_host) {
  if (!op || k <= 0 || k > 4096 || !eig_host || !mu || !occ_host || !(kT > 0) || max_iter < 1)
    return TTG_BAD_ARG;
  double* e = op->scal.as<double>() + kScalEig;
  double* out = op->scal.as<double>() + kScalFermi;
  double* occ = op->kk2.as<double>();
  TTG_CUDA_TRY(cudaMemcpyAsync(e, eig_host, (size_t)k * 8, cudaMemcpyHostToDevice, op->stream));
  TTG_TRY(fermi(op, e, k, n_electrons, kT, max_iter, occ, out));
  double res[3];
  TTG_CUDA_TRY(cudaMemcpyAsync(res, out, 24, cudaMemcpyDeviceToHost, op->stream));
  TTG_CUDA_TRY(cudaMemcpyAsync(occ_host, occ, (size_t)k * 8, cudaMemcpyDeviceToHost, op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  *mu = res[0];
  return res[2] <= 1e-8 ? TTG_OK : TTG_NOT_CONVERGED;
}

}  // extern "C"
