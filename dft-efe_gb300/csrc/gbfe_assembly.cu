// gbfe_assembly.cu -- the two steps either side of the eigensolve:
//
// * cell-matrix assembly, A_c = alpha * F_c + B_c^T diag(w_c) B_c:
//   the reference's KohnShamOperatorContextFE::reinit
//   (ksdft/KohnShamOperatorContextFE.t.cpp:1253-1311) summing the kinetic part
//   0.5 grad N_i . grad N_j (ksdft/KineticFE.t.cpp:90-97, F_c here) and the local
//   potential part int N_i V N_j (ksdft/ElectrostaticLocalFE.t.cpp:1625-1660:
//   w_c(q) = JxW_c(q) V(x_cq), B_c the basis values at the cell's quadrature
//   points).  Cells may differ in size and quadrature (enriched cells carry
//   extra basis functions and a finer rule); a uniform mesh shares one B.
//   FP64 on the CUDA cores: per (cell, 64 x 64 output tile pair) a CTA streams
//   16 quadrature points at a time through shared memory, each thread owns a
//   4 x 4 block of the tile; only the upper triangle is computed and mirrored,
//   so every A_c is exactly symmetric.  The derived copies (FP32, split-BF16
//   tiles, FP64 slices) are rebuilt.
// * electron density, rho_c(q) = sum_i 2 f_i psi_i(x_cq)^2 with
//   psi_i(x_cq) = sum_a B_c[q][a] Psi[ids_c[a]][i]
//   (ksdft/DensityCalculator.t.cpp:37-100 and :283-345, interpolation then the
//   occupation-weighted square, spin factor 2), two routes:
//   - gbfe_density_cells: FP64 CUDA cores, any cell sizes and rules; per
//     (cell, 64-vector tile) the gathered Psi tile sits in shared memory, a
//     thread per quadrature point; partial sums per vector tile are added in
//     tile order (deterministic);
//   - gbfe_density_op: the interpolation B_c Psi_c is a cell product with
//     B_c as the cell's "matrix" (quadrature point q in place of the output
//     dof, so nq_c = nd_c), run by the operator's FP64 cell product -- the
//     sliced FP64-accurate tensor-core kernel when the operator carries the
//     slices and the context's FP64 mode selects it -- then the
//     occupation-weighted squares are summed per point by one warp in a fixed
//     order.
#include "gbfe_internal.cuh"

#include <algorithm>
#include <vector>

using namespace gbfe;

namespace {

constexpr uint32_t AT = 64;  // assembly output tile
constexpr uint32_t AQ = 16;  // quadrature points per shared-memory chunk

// grid (cell, upper-triangle tile pair); block 256 = 16 x 16 threads of 4 x 4
__global__ void __launch_bounds__(256) k_assemble_cells(const double *__restrict__ B, const uint64_t *__restrict__ b_off,
                                                        const uint64_t *__restrict__ q_off,
                                                        const double *__restrict__ w,
                                                        const uint32_t *__restrict__ cell_off,
                                                        const double *__restrict__ fixed, double alpha,
                                                        const uint64_t *__restrict__ mat_off, double *__restrict__ mats) {
  __shared__ double Bi[AQ][AT], Bj[AQ][AT];
  const uint32_t c = blockIdx.x;
  const uint32_t nd = cell_off[c + 1] - cell_off[c];
  const uint32_t nt = (nd + AT - 1) / AT;
  uint32_t p = blockIdx.y, ti = 0;
  while (ti < nt && p >= nt - ti) {
    p -= nt - ti;
    ++ti;
  }
  if (ti >= nt) return;  // a pair beyond this cell's tiles
  const uint32_t tj = ti + p;
  const uint32_t tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const uint64_t q0c = q_off[c];
  const uint32_t nq = (uint32_t)(q_off[c + 1] - q0c);
  const double *Bc = B + b_off[c];
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) acc[r][s] = 0.0;
  for (uint32_t q0 = 0; q0 < nq; q0 += AQ) {
    for (uint32_t t = threadIdx.x; t < AQ * AT; t += blockDim.x) {
      const uint32_t qq = t / AT, a = t % AT, q = q0 + qq;
      const uint32_t ii = ti * AT + a, jj = tj * AT + a;
      const bool qin = q < nq;
      Bi[qq][a] = (qin && ii < nd) ? Bc[(uint64_t)q * nd + ii] * w[q0c + q] : 0.0;
      Bj[qq][a] = (qin && jj < nd) ? Bc[(uint64_t)q * nd + jj] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (uint32_t qq = 0; qq < AQ; ++qq) {
      double bi[4], bj[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) bi[r] = Bi[qq][ty * 4 + r];
#pragma unroll
      for (int s = 0; s < 4; ++s) bj[s] = Bj[qq][tx * 4 + s];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) acc[r][s] = fma(bi[r], bj[s], acc[r][s]);
    }
    __syncthreads();
  }
  const uint64_t base = mat_off[c];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const uint32_t i = ti * AT + ty * 4 + r, j = tj * AT + tx * 4 + s;
      if (i < nd && j < nd && i <= j) {
        const double fij = fixed ? fixed[base + i + (uint64_t)nd * j] : 0.0;
        mats[base + i + (uint64_t)nd * j] = alpha * fij + acc[r][s];
        if (i != j) {
          const double fji = fixed ? fixed[base + j + (uint64_t)nd * i] : 0.0;
          mats[base + j + (uint64_t)nd * i] = alpha * fji + acc[r][s];
        }
      }
    }
}

constexpr uint32_t DV = 64;  // density: vectors per CTA

// grid (cell, vector tile); part[tile][point] = sum over the tile's vectors
__global__ void __launch_bounds__(256) k_density_cells(const double *__restrict__ Psi, uint32_t m,
                                                       const uint32_t *__restrict__ ids,
                                                       const uint32_t *__restrict__ cell_off,
                                                       const double *__restrict__ B, const uint64_t *__restrict__ b_off,
                                                       const uint64_t *__restrict__ q_off,
                                                       const double *__restrict__ occ, uint64_t nq_total,
                                                       double *__restrict__ part) {
  extern __shared__ double psh[];  // [nd][DV]
  const uint32_t c = blockIdx.x, v0 = blockIdx.y * DV;
  const uint32_t nv = min(DV, m - v0);
  const uint32_t off = cell_off[c], nd = cell_off[c + 1] - off;
  for (uint32_t idx = threadIdx.x; idx < nd * DV; idx += blockDim.x) {
    const uint32_t a = idx / DV, i = idx - a * DV;
    psh[idx] = i < nv ? Psi[(uint64_t)ids[off + a] * m + v0 + i] : 0.0;
  }
  __syncthreads();
  const uint64_t q0c = q_off[c];
  const uint32_t nq = (uint32_t)(q_off[c + 1] - q0c);
  const double *Bc = B + b_off[c];
  for (uint32_t q = threadIdx.x; q < nq; q += blockDim.x) {
    const double *Bq = Bc + (uint64_t)q * nd;
    double r = 0.0;
    for (uint32_t i0 = 0; i0 < nv; i0 += 16) {
      double psi[16];
#pragma unroll
      for (int ii = 0; ii < 16; ++ii) psi[ii] = 0.0;
      for (uint32_t a = 0; a < nd; ++a) {
        const double b = __ldg(Bq + a);
#pragma unroll
        for (int ii = 0; ii < 16; ++ii) psi[ii] = fma(b, psh[a * DV + i0 + ii], psi[ii]);
      }
#pragma unroll
      for (int ii = 0; ii < 16; ++ii)
        if (i0 + ii < nv) r += 2.0 * psi[ii] * psi[ii] * occ[v0 + i0 + ii];
    }
    part[(uint64_t)blockIdx.y * nq_total + q0c + q] = r;
  }
}

__global__ void k_density_sum_tiles(const double *__restrict__ part, uint32_t tiles, uint64_t n,
                                    double *__restrict__ rho) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (uint32_t k = 0; k < tiles; ++k) s += part[(uint64_t)k * n + t];
    rho[t] = s;
  }
}

// rho[t] = sum_i 2 f_i Yc[t][i]^2: one warp per point, lane i, i + 32, ...,
// then a fixed shuffle tree (deterministic)
__global__ void k_density_rows(const double *__restrict__ Yc, uint32_t m, uint64_t rows,
                               const double *__restrict__ occ, double *__restrict__ rho) {
  const uint32_t lane = threadIdx.x % 32;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t t = blockIdx.x * (uint64_t)(blockDim.x / 32) + threadIdx.x / 32; t < rows; t += nw) {
    double r = 0.0;
    for (uint32_t i = lane; i < m; i += 32) {
      const double y = Yc[t * m + i];
      r += 2.0 * y * y * occ[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0) rho[t] = r;
  }
}

__global__ void k_f64_to_f32_mats(const double *__restrict__ s, float *__restrict__ d, uint64_t n) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    d[t] = (float)s[t];
}

// per-cell offsets into the basis table and the quadrature points: a shared
// table (nq_per_cell == nullptr: every cell has nq points, one B) or one
// nq_c x nd_c block per cell
void quad_layout(const gbfe_mesh *me, uint32_t nq, const uint32_t *nq_per_cell, std::vector<uint64_t> &b_off,
                 std::vector<uint64_t> &q_off) {
  b_off.assign(me->n_cells, 0);
  q_off.assign(me->n_cells + 1, 0);
  uint64_t b = 0;
  for (uint32_t c = 0; c < me->n_cells; ++c) {
    const uint32_t nqc = nq_per_cell ? nq_per_cell[c] : nq;
    GBFE_REQUIRE(nqc > 0, "quadrature: a cell with no points");
    q_off[c + 1] = q_off[c] + nqc;
    if (nq_per_cell) {
      b_off[c] = b;
      b += (uint64_t)nqc * me->h_nd[c];
    }
  }
}

uint64_t table_size(const gbfe_mesh *me, uint32_t nq, const uint32_t *nq_per_cell) {
  if (!nq_per_cell) return (uint64_t)nq * me->nd_max;
  uint64_t b = 0;
  for (uint32_t c = 0; c < me->n_cells; ++c) b += (uint64_t)nq_per_cell[c] * me->h_nd[c];
  return b;
}

void assemble_impl(gbfe_op *op, uint32_t nq, const uint32_t *nq_per_cell, const double *basis_values,
                   const double *weights, const double *fixed_mats, double alpha) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  GBFE_REQUIRE(op->kind == OP_CELL && !op->mat_off_own.p, "assemble: needs a per-cell matrix operator");
  GBFE_REQUIRE(nq_per_cell || me->nd_min == me->nd_max, "assemble: one shared basis table needs cells of one size");
  std::vector<uint64_t> bo, qo;
  quad_layout(me, nq, nq_per_cell, bo, qo);
  DBuf<double> B, w, F;
  DBuf<uint64_t> b_off, q_off;
  B.upload(basis_values, table_size(me, nq, nq_per_cell), ctx->stream);
  w.upload(weights, qo.back(), ctx->stream);
  b_off.upload(bo.data(), bo.size(), ctx->stream);
  q_off.upload(qo.data(), qo.size(), ctx->stream);
  if (fixed_mats) F.upload(fixed_mats, me->total_mat, ctx->stream);
  const uint32_t nt = (me->nd_max + AT - 1) / AT;
  k_assemble_cells<<<dim3(me->n_cells, nt * (nt + 1) / 2), 256, 0, ctx->stream>>>(
      B.p, b_off.p, q_off.p, w.p, me->cell_off.p, fixed_mats ? F.p : nullptr, alpha, me->mat_off.p, op->mats.p);
  check_launch(ctx, "assemble_cells");
  // derived copies follow the new FP64 matrices
  if (op->mats_f32.p) {
    const uint64_t n = op->mats_count;
    unsigned g = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
    k_f64_to_f32_mats<<<g ? g : 1, 256, 0, ctx->stream>>>(op->mats.p, op->mats_f32.p, n);
    check_launch(ctx, "f64_to_f32");
  }
  if (op->tc_aoff.p) build_tc_mats(op);
  op->folded_for = 0;  // folded tiles follow the new matrices on their next use
  if (op->oz_aoff.p) build_oz_mats(op);
  GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
}

void density_impl(const gbfe_mv *Psi, const double *occupation, uint32_t nq, const uint32_t *nq_per_cell,
                  const double *basis_values, double *rho_host) {
  gbfe_mesh *me = Psi->mesh;
  gbfe_ctx *ctx = me->ctx;
  GBFE_REQUIRE(Psi->dtype == GBFE_F64, "density: Psi must be FP64");
  GBFE_REQUIRE(nq_per_cell || me->nd_min == me->nd_max, "density: one shared basis table needs cells of one size");
  const uint32_t m = Psi->m;
  GBFE_REQUIRE(m > 0, "density: no vectors");
  const size_t smem = sizeof(double) * (size_t)me->nd_max * DV;
  GBFE_REQUIRE(smem <= 200 * 1024, "density: cells above 400 dofs are not supported");
  static PerDeviceOnce attr_once;
  attr_once.run(ctx->device, [&] {
    GBFE_CUDA(cudaFuncSetAttribute(k_density_cells, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  });
  std::vector<uint64_t> bo, qo;
  quad_layout(me, nq, nq_per_cell, bo, qo);
  const uint64_t npts = qo.back();
  const uint32_t tiles = (m + DV - 1) / DV;
  DBuf<double> B, occ, part, rho;
  DBuf<uint64_t> b_off, q_off;
  B.upload(basis_values, table_size(me, nq, nq_per_cell), ctx->stream);
  occ.upload(occupation, m, ctx->stream);
  b_off.upload(bo.data(), bo.size(), ctx->stream);
  q_off.upload(qo.data(), qo.size(), ctx->stream);
  part.alloc((size_t)tiles * npts);
  rho.alloc(npts);
  k_density_cells<<<dim3(me->n_cells, tiles), 256, smem, ctx->stream>>>(Psi->d.p, m, me->ids.p, me->cell_off.p, B.p,
                                                                        b_off.p, q_off.p, occ.p, npts, part.p);
  check_launch(ctx, "density_cells");
  k_density_sum_tiles<<<(unsigned)std::min<uint64_t>((npts + 255) / 256, (uint64_t)ctx->sm_count * 8), 256, 0,
                        ctx->stream>>>(part.p, tiles, npts, rho.p);
  check_launch(ctx, "density_sum_tiles");
  GBFE_CUDA(cudaMemcpyAsync(rho_host, rho.p, npts * 8, cudaMemcpyDeviceToHost, ctx->stream));
  GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace

extern "C" {

int gbfe_op_assemble_local(gbfe_op *op, uint32_t nq, const double *basis_values, const double *weights,
                           const double *fixed_mats, double alpha) {
  if (!op || !basis_values || !weights || nq == 0) return GBFE_ERR_ARG;
  return gbfe_guard(op->mesh->ctx, [&] { assemble_impl(op, nq, nullptr, basis_values, weights, fixed_mats, alpha); });
}

int gbfe_op_assemble_cells(gbfe_op *op, const uint32_t *nq_per_cell, const double *basis_values,
                           const double *weights, const double *fixed_mats, double alpha) {
  if (!op || !nq_per_cell || !basis_values || !weights) return GBFE_ERR_ARG;
  return gbfe_guard(op->mesh->ctx,
                    [&] { assemble_impl(op, 0, nq_per_cell, basis_values, weights, fixed_mats, alpha); });
}

int gbfe_density(const gbfe_mv *Psi, const double *occupation, uint32_t nq, const double *basis_values,
                 double *rho_host) {
  if (!Psi || !occupation || !basis_values || !rho_host || nq == 0) return GBFE_ERR_ARG;
  return gbfe_guard(Psi->mesh->ctx, [&] { density_impl(Psi, occupation, nq, nullptr, basis_values, rho_host); });
}

int gbfe_density_cells(const gbfe_mv *Psi, const double *occupation, const uint32_t *nq_per_cell,
                       const double *basis_values, double *rho_host) {
  if (!Psi || !occupation || !nq_per_cell || !basis_values || !rho_host) return GBFE_ERR_ARG;
  return gbfe_guard(Psi->mesh->ctx, [&] { density_impl(Psi, occupation, 0, nq_per_cell, basis_values, rho_host); });
}

int gbfe_density_op(const gbfe_op *basis_op, gbfe_mv *Psi, const double *occupation, double *rho_host) {
  if (!basis_op || !Psi || !occupation || !rho_host) return GBFE_ERR_ARG;
  gbfe_mesh *me = Psi->mesh;
  gbfe_ctx *ctx = me->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(basis_op->mesh == me && basis_op->kind == OP_CELL && !basis_op->cons && !basis_op->nl,
                 "density_op: needs a cell operator of Psi's mesh built without constraints");
    GBFE_REQUIRE(Psi->dtype == GBFE_F64 && Psi->m > 0, "density_op: Psi must be FP64 with vectors");
    const uint32_t m = Psi->m;
    DBuf<double> Yc, occ, rho;
    Yc.alloc((size_t)me->total_cell_dofs * m);
    occ.upload(occupation, m, ctx->stream);
    rho.alloc(me->total_cell_dofs);
    cell_product_f64(basis_op, Psi, Yc.p);
    k_density_rows<<<(unsigned)std::min<uint64_t>((me->total_cell_dofs + 7) / 8, (uint64_t)ctx->sm_count * 16), 256, 0,
                     ctx->stream>>>(Yc.p, m, me->total_cell_dofs, occ.p, rho.p);
    check_launch(ctx, "density_rows");
    GBFE_CUDA(cudaMemcpyAsync(rho_host, rho.p, me->total_cell_dofs * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

}  // extern "C"
