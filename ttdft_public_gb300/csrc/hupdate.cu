// New values of H_loc for a new effective potential, on the device.
//
// The reference rebuilds H_loc on the host every SCF iteration
// (ProjectHamiltonianSparse::Create_Hloc, dft/ProjectHamiltonianSparse.cc:
// 330-575, called from main.cc:965-972): for row I = (xI, yI, zI) and column
// J = (xJ, yJ, zJ)
//   H[I,J] = 0.5 (DX MY MZ + MX DY MZ + MX MY DZ)[I,J]
//          + sum_abc G_abc PX_a[xI,xJ] PY_b[yI,yJ] PZ_c[zI,zJ]
// with V_eff = sum_abc G_abc u_a(x) v_b(y) w_c(z) its Tucker decomposition
// (main.cc:951-955) and PX_a[i,j] = int psi_i u_a psi_j.
//
// Here the sparsity pattern is the one fixed when the operator was created,
// and the values are recomputed in place: the Tucker sum is factorised
// through (x-pair, y-pair) intermediates
//   T1[b][xp][c]     = sum_a PX_a[xp] G_abc                  (batched FP64 GEMM)
//   T2[yp][xp][c]    = sum_b PY_b[yp] T1[b][xp][c]           (one FP64 GEMM)
//   H_pot[I,J]       = sum_c PZ_c[zp] T2[yp][xp][c]          (per entry, r_c FMAs)
// and each new value is written straight into every device format through
// the position maps recorded when the formats were packed.  FP64 throughout.

#include <algorithm>
#include <cmath>
#include <vector>

#include "ttg_internal.cuh"

namespace ttg {
namespace {

struct UpdateArgs {
  const int64_t* row_ptr;
  const int* col;
  const int* rg_pos;
  const int* tile_base;
  const uint8_t* tile_slot;
  int rx, ry, rz;
  int bw[3];                  // half-bandwidths of the pair tables
  const double* kin;          // DX DY DZ MX MY MZ, each r_d x r_d row-major
  const double* T2;           // [yp][xp][c]
  const double* PZp;          // [zp][c]
  int rc;                     // Tucker rank of the potential along z
  int64_t nxp;
  double* v64;
  float2* vdf;
  float* v32;
  __nv_bfloat16* v16;
  float* t32;
  __nv_bfloat16* t16;
  const int64_t* rg_gptr;     // slot offset of each row group
  const int* umma_pos;        // slot of the entry within its 128-row tile
  const int* umma_row;        // tile * 128 + lane of each row
  const int64_t* umma_tptr;   // slot offset of each tile (multiples of 16)
  __nv_bfloat16* u16;         // the tiles' three BF16 planes (2048 elements apart)
  int64_t n;
};

__device__ __forceinline__ int pair_index(int i, int j, int bw) {
  const int d = j - i;
  return (d < -bw || d > bw) ? -1 : i * (2 * bw + 1) + d + bw;
}

__global__ void k_update_values(UpdateArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= a.n) return;
  const int xI = (int)(row % a.rx);
  const int yI = (int)((row / a.rx) % a.ry);
  const int zI = (int)(row / ((int64_t)a.rx * a.ry));
  const int rx = a.rx, ry = a.ry, rz = a.rz;
  const double* DX = a.kin;
  const double* DY = DX + rx * rx;
  const double* DZ = DY + ry * ry;
  const double* MX = DZ + rz * rz;
  const double* MY = MX + rx * rx;
  const double* MZ = MY + ry * ry;
  for (int64_t e = a.row_ptr[row] + lane; e < a.row_ptr[row + 1]; e += 32) {
    const int J = a.col[e];
    const int xJ = J % rx, yJ = (J / rx) % ry, zJ = J / (rx * ry);
    const double dx = DX[xI * rx + xJ], mx = MX[xI * rx + xJ];
    const double dy = DY[yI * ry + yJ], my = MY[yI * ry + yJ];
    const double dz = DZ[zI * rz + zJ], mz = MZ[zI * rz + zJ];
    double val = 0.5 * (dx * my * mz + mx * dy * mz + mx * my * dz);
    const int xp = pair_index(xI, xJ, a.bw[0]);
    const int yp = pair_index(yI, yJ, a.bw[1]);
    const int zp = pair_index(zI, zJ, a.bw[2]);
    if (xp >= 0 && yp >= 0 && zp >= 0) {
      const double* t2 = a.T2 + ((int64_t)yp * a.nxp + xp) * a.rc;
      const double* pz = a.PZp + (int64_t)zp * a.rc;
      // four independent partial sums: the FP64 FMA chain of one sum would
      // otherwise serialise the rc terms of every entry
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      int c = 0;
      for (; c + 3 < a.rc; c += 4) {
        s0 = fma(pz[c], t2[c], s0);
        s1 = fma(pz[c + 1], t2[c + 1], s1);
        s2 = fma(pz[c + 2], t2[c + 2], s2);
        s3 = fma(pz[c + 3], t2[c + 3], s3);
      }
      for (; c < a.rc; ++c) s0 = fma(pz[c], t2[c], s0);
      val += (s0 + s1) + (s2 + s3);
    }
    // value index in the row groups: (group slot offset + slot) * 8 + row in group
    const int64_t p = (a.rg_gptr[row >> 3] + a.rg_pos[e]) * 8 + (row & 7);
    a.v64[p] = val;
    if (a.vdf) {
      const float h = __double2float_rn(val);
      a.vdf[p] = make_float2(h, __double2float_rn(val - (double)h));
    }
    if (a.v32) a.v32[p] = (float)val;
    if (a.v16) a.v16[p] = __double2bfloat16(val);
    if (a.t32) {
      // fragment order of spmm_tc.cu: TF32 lane 4g+(j%4), element j/4;
      // BF16 lane 4g+((j%8)/2), element (j%2) + 2*(j/8)
      const int base = a.tile_base[e];
      const int j = a.tile_slot[e];
      a.t32[(int64_t)(base + (j & 3)) * 4 + (j >> 2)] = (float)val;
      a.t16[(int64_t)(base + ((j & 7) >> 1)) * 4 + (j & 1) + 2 * (j >> 3)] = __double2bfloat16(val);
    }
    if (a.u16) {
      // three BF16 terms, as the tile builder splits them
      // element in plane 0: chunk (tile's first + slot / 16), canonical K-major
      // position of (lane, slot % 16) within the chunk's 128 x 16 plane
      const int ur = a.umma_row[row];
      const int m = ur & 127, sl = a.umma_pos[e];
      const int64_t chunk = a.umma_tptr[ur >> 7] / 16 + (sl >> 4);
      const int s16 = sl & 15;
      __nv_bfloat16* u = a.u16 + chunk * 6144 + ((m >> 3) * 128 + (s16 >> 3) * 64 + (m & 7) * 8 +
                                                 (s16 & 7));
      const __nv_bfloat16 h0 = __float2bfloat16_rn((float)val);
      const double r1 = val - (double)__bfloat162float(h0);
      const __nv_bfloat16 h1 = __float2bfloat16_rn((float)r1);
      u[0] = h0;
      u[2048] = h1;
      u[4096] = __float2bfloat16_rn((float)(r1 - (double)__bfloat162float(h1)));
    }
  }
}

}  // namespace
}  // namespace ttg

using namespace ttg;

namespace ttg {
namespace {

// pair tables PXp[xp][a] = PX_a[i][j], xp = i (2b + 1) + (j - i) + b, from
// the (rk x r x r) row-major matrices on the device
__global__ void k_pair_table(const double* __restrict__ pm, int r, int rk, int b,
                             double* __restrict__ out) {
  const int64_t np = (int64_t)r * (2 * b + 1);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < np * rk;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / rk;
    const int a = (int)(e - p * rk);
    const int i = (int)(p / (2 * b + 1));
    const int j = i + (int)(p - (int64_t)i * (2 * b + 1)) - b;
    out[e] = (j >= 0 && j < r) ? pm[((int64_t)a * r + i) * r + j] : 0.0;
  }
}

struct UpdateLayout {
  int ra, rb, rc;
  int64_t nxp, nyp, nzp, off_x, off_y, off_z, off_g, off_t1, off_t2, total;
};

ttg_status update_layout(ttg_op* op, const int32_t* pot_ranks, UpdateLayout& L) {
  Pattern& P = op->pattern;
  L.ra = pot_ranks[0];
  L.rb = pot_ranks[1];
  L.rc = pot_ranks[2];
  if (L.ra <= 0 || L.rb <= 0 || L.rc <= 0) return TTG_BAD_ARG;
  L.nxp = (int64_t)P.r[0] * (2 * P.bw[0] + 1);
  L.nyp = (int64_t)P.r[1] * (2 * P.bw[1] + 1);
  L.nzp = (int64_t)P.r[2] * (2 * P.bw[2] + 1);
  const int64_t ncore = (int64_t)L.ra * L.rb * L.rc;
  L.off_x = 0;
  L.off_y = L.off_x + L.nxp * L.ra;
  L.off_z = L.off_y + L.nyp * L.rb;
  L.off_g = L.off_z + L.nzp * L.rc;
  L.off_t1 = L.off_g + ncore;
  L.off_t2 = L.off_t1 + L.nxp * L.rb * L.rc;
  L.total = L.off_t2 + L.nyp * L.nxp * L.rc;
  if ((int64_t)P.work.bytes < L.total * 8) TTG_TRY(P.work.alloc(L.total * 8));
  return TTG_OK;
}

// T1, T2 and the per-entry update, from the pair tables and the core in work
ttg_status update_from_tables(ttg_op* op, const UpdateLayout& L) {
  Pattern& P = op->pattern;
  const int rx = P.r[0], ry = P.r[1], rz = P.r[2];
  const int ra = L.ra, rb = L.rb, rc = L.rc;
  const int bw[3] = {P.bw[0], P.bw[1], P.bw[2]};
  const int64_t nxp = L.nxp, nyp = L.nyp;
  const int64_t off_x = L.off_x, off_y = L.off_y, off_z = L.off_z, off_g = L.off_g,
                off_t1 = L.off_t1, off_t2 = L.off_t2;
  double* w = P.work.as<double>();
  cudaStream_t st = op->stream;
  // T1[b][xp][c] = sum_a PXp[xp][a] G[a + ra (b + rb c)]   (batch over b)
  TTG_TRY(dgemm(st, (int)nxp, rc, ra, rb, DOp{w + off_x, ra, 1, 0},
                DOp{w + off_g, 1, (int64_t)ra * rb, ra}, w + off_t1, rc, 1, nxp * rc, P.work2));
  // T2[yp][(xp, c)] = sum_b PYp[yp][b] T1[b][(xp, c)]: one GEMM, N = nxp * rc
  TTG_TRY(dgemm(st, (int)nyp, (int)(nxp * rc), rb, 1, DOp{w + off_y, rb, 1, 0},
                DOp{w + off_t1, nxp * rc, 1, 0}, w + off_t2, nxp * rc, 1, 0, P.work2));
  UpdateArgs a{};
  a.row_ptr = P.row_ptr.as<int64_t>();
  a.col = P.col.as<int>();
  a.rg_pos = P.rg_pos.as<int>();
  a.tile_base = P.tile_base.as<int>();
  a.tile_slot = P.tile_slot.as<uint8_t>();
  a.rx = rx;
  a.ry = ry;
  a.rz = rz;
  for (int d = 0; d < 3; ++d) a.bw[d] = bw[d];
  a.kin = P.kin.as<double>();
  a.T2 = w + off_t2;
  a.PZp = w + off_z;
  a.rc = rc;
  a.nxp = nxp;
  a.v64 = op->rg.v64.as<double>();
  a.vdf = op->rg.vdf.as<float2>();
  a.v32 = op->rg.v32.as<float>();
  a.v16 = op->rg.v16.as<__nv_bfloat16>();
  a.t32 = op->tiles.n_tiles > 0 && P.tile_base.p ? op->tiles.v32.as<float>() : nullptr;
  a.t16 = op->tiles.v16.as<__nv_bfloat16>();
  a.rg_gptr = op->rg.gptr.as<int64_t>();
  a.umma_pos = P.umma_pos.as<int>();
  a.umma_row = P.umma_row.as<int>();
  a.umma_tptr = op->umma.tptr.as<int64_t>();
  a.u16 = op->umma.n_tiles > 0 && P.umma_pos.p ? op->umma.hpl.as<__nv_bfloat16>() : nullptr;
  a.n = op->n;
  const int wpb = 8;
  k_update_values<<<(unsigned)((op->n + wpb - 1) / wpb), 32 * wpb, 0, st>>>(a); TTG_COUNT();
  TTG_LAUNCHED(op);
  return TTG_OK;
}

}  // namespace
}  // namespace ttg


extern "C" {

ttg_status ttg_op_set_kinetic(ttg_op* op, const double* dx, const double* dy, const double* dz,
                              const double* mx, const double* my, const double* mz) {
  if (!op || !op->keep_pattern || !dx || !dy || !dz || !mx || !my || !mz) return TTG_BAD_ARG;
  Pattern& P = op->pattern;
  const int rx = P.r[0], ry = P.r[1], rz = P.r[2];
  const size_t cnt = 2 * ((size_t)rx * rx + (size_t)ry * ry + (size_t)rz * rz);
  if (!P.kin.p) TTG_TRY(P.kin.alloc(cnt * 8));
  std::vector<double> h;
  h.reserve(cnt);
  h.insert(h.end(), dx, dx + rx * rx);
  h.insert(h.end(), dy, dy + ry * ry);
  h.insert(h.end(), dz, dz + rz * rz);
  h.insert(h.end(), mx, mx + rx * rx);
  h.insert(h.end(), my, my + ry * ry);
  h.insert(h.end(), mz, mz + rz * rz);
  TTG_CUDA_TRY(cudaMemcpyAsync(P.kin.p, h.data(), cnt * 8, cudaMemcpyHostToDevice, op->stream));
  TTG_CUDA_TRY(cudaStreamSynchronize(op->stream));
  P.kinetic_set = true;
  return TTG_OK;
}

ttg_status ttg_op_update_potential(ttg_op* op, const int32_t* pot_ranks, const double* G,
                                   const double* px, const double* py, const double* pz) {
  if (!op || !op->keep_pattern || !op->pattern.kinetic_set || !pot_ranks || !G || !px || !py ||
      !pz)
    return TTG_BAD_ARG;
  Pattern& P = op->pattern;
  UpdateLayout L;
  TTG_TRY(update_layout(op, pot_ranks, L));
  // pair tables PXp[xp][a] = PX_a[i][j] (host: O(pairs * rank))
  auto pairs = [](const double* pm, int r, int rk, int b, std::vector<double>& out) {
    const int64_t np = (int64_t)r * (2 * b + 1);
    out.assign(np * rk, 0.0);
    for (int i = 0; i < r; ++i)
      for (int d = -b; d <= b; ++d) {
        const int j = i + d;
        if (j < 0 || j >= r) continue;
        const int64_t p = (int64_t)i * (2 * b + 1) + d + b;
        for (int a = 0; a < rk; ++a) out[p * rk + a] = pm[((int64_t)a * r + i) * r + j];
      }
  };
  std::vector<double> hx, hy, hz;
  pairs(px, P.r[0], L.ra, P.bw[0], hx);
  pairs(py, P.r[1], L.rb, P.bw[1], hy);
  pairs(pz, P.r[2], L.rc, P.bw[2], hz);
  double* w = P.work.as<double>();
  cudaStream_t st = op->stream;
  const int64_t ncore = (int64_t)L.ra * L.rb * L.rc;
  TTG_CUDA_TRY(cudaMemcpyAsync(w + L.off_x, hx.data(), hx.size() * 8, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(w + L.off_y, hy.data(), hy.size() * 8, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(w + L.off_z, hz.data(), hz.size() * 8, cudaMemcpyHostToDevice, st));
  TTG_CUDA_TRY(cudaMemcpyAsync(w + L.off_g, G, ncore * 8, cudaMemcpyHostToDevice, st));
  TTG_TRY(update_from_tables(op, L));
  TTG_CUDA_TRY(cudaStreamSynchronize(st));
  return TTG_OK;
}

ttg_status ttg_op_update_potential_device(ttg_op* op, const int32_t* pot_ranks,
                                          const double* g_dev, const double* px_dev,
                                          const double* py_dev, const double* pz_dev) {
  if (!op || !op->keep_pattern || !op->pattern.kinetic_set || !pot_ranks || !g_dev || !px_dev ||
      !py_dev || !pz_dev)
    return TTG_BAD_ARG;
  Pattern& P = op->pattern;
  UpdateLayout L;
  TTG_TRY(update_layout(op, pot_ranks, L));
  double* w = P.work.as<double>();
  cudaStream_t st = op->stream;
  const double* pm[3] = {px_dev, py_dev, pz_dev};
  const int rk[3] = {L.ra, L.rb, L.rc};
  const int64_t off[3] = {L.off_x, L.off_y, L.off_z};
  const int64_t np[3] = {L.nxp, L.nyp, L.nzp};
  for (int d = 0; d < 3; ++d) {
    const int64_t n = np[d] * rk[d];
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    k_pair_table<<<std::max(blocks, 1), 256, 0, st>>>(pm[d], P.r[d], rk[d], P.bw[d], w + off[d]); TTG_COUNT();
    TTG_LAUNCHED(op);
  }
  TTG_CUDA_TRY(cudaMemcpyAsync(w + L.off_g, g_dev, (size_t)L.ra * L.rb * L.rc * 8,
                               cudaMemcpyDeviceToDevice, st));
  return update_from_tables(op, L);
}

}  // extern "C"
