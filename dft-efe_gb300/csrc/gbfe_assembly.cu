// gbfe_assembly.cu -- the two steps either side of the eigensolve:
//
// * gbfe_op_assemble_local: rebuild a cell operator's matrices on the device,
//     A_c = alpha * F_c + B^T diag(w_c) B,
//   the reference's KohnShamOperatorContextFE::reinit
//   (ksdft/KohnShamOperatorContextFE.t.cpp:1253-1311) summing the kinetic part
//   0.5 grad N_i . grad N_j (ksdft/KineticFE.t.cpp:90-97, F_c here) and the local
//   potential part int N_i V N_j (ksdft/ElectrostaticLocalFE.t.cpp:1625-1660:
//   w_c(q) = JxW_c(q) V(x_cq), B the basis values at the quadrature points).
//   The derived copies (FP32, split-BF16 tiles, FP64 slices) are rebuilt.
// * gbfe_density: rho_c(q) = sum_i 2 f_i psi_i(x_cq)^2 with
//   psi_i(x_cq) = sum_a B[q][a] Psi[ids_c[a]][i]
//   (ksdft/DensityCalculator.t.cpp:37-100 and :283-345, interpolation then the
//   occupation-weighted square, spin factor 2).
// Both need cells of one size (uniform nd) and run in FP64.
#include "gbfe_internal.cuh"

#include <algorithm>

using namespace gbfe;

namespace {

// one CTA per cell; threads over the upper triangle (i <= j)
__global__ void k_assemble_local(const double *__restrict__ B, uint32_t nq, uint32_t nd,
                                 const double *__restrict__ w, const double *__restrict__ fixed, double alpha,
                                 const uint64_t *__restrict__ mat_off, double *__restrict__ mats) {
  extern __shared__ double wsh[];
  const uint32_t c = blockIdx.x;
  for (uint32_t q = threadIdx.x; q < nq; q += blockDim.x) wsh[q] = w[(uint64_t)c * nq + q];
  __syncthreads();
  const uint64_t base = mat_off[c];
  const uint32_t npair = nd * (nd + 1) / 2;
  for (uint32_t t = threadIdx.x; t < npair; t += blockDim.x) {
    // t -> (i, j), j >= i, column-major upper triangle enumeration
    uint32_t j = (uint32_t)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((j + 1) * (j + 2) / 2 <= t) ++j;
    while (j * (j + 1) / 2 > t) --j;
    const uint32_t i = t - j * (j + 1) / 2;
    double acc = 0.0;
    for (uint32_t q = 0; q < nq; ++q) acc = fma(B[(uint64_t)q * nd + i] * wsh[q], B[(uint64_t)q * nd + j], acc);
    const double fij = fixed ? fixed[base + i + (uint64_t)nd * j] : 0.0;
    const double fji = fixed ? fixed[base + j + (uint64_t)nd * i] : 0.0;
    mats[base + i + (uint64_t)nd * j] = alpha * fij + acc;
    if (i != j) mats[base + j + (uint64_t)nd * i] = alpha * fji + acc;
  }
}

// one CTA per cell; Psi_c gathered into shared memory; threads over quadrature points
__global__ void k_density(const double *__restrict__ Psi, uint32_t m, const uint32_t *__restrict__ ids,
                          const uint32_t *__restrict__ cell_off, const double *__restrict__ B, uint32_t nq,
                          const double *__restrict__ occ, double *__restrict__ rho) {
  extern __shared__ double psh[];
  const uint32_t c = blockIdx.x;
  const uint32_t off = cell_off[c], nd = cell_off[c + 1] - off;
  for (uint32_t idx = threadIdx.x; idx < nd * m; idx += blockDim.x) {
    const uint32_t a = idx / m, i = idx - a * m;
    psh[idx] = Psi[(uint64_t)ids[off + a] * m + i];
  }
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < nq; q += blockDim.x) {
    double r = 0.0;
    for (uint32_t i = 0; i < m; ++i) {
      double psi = 0.0;
      for (uint32_t a = 0; a < nd; ++a) psi = fma(B[(uint64_t)q * nd + a], psh[a * m + i], psi);
      r += 2.0 * psi * psi * occ[i];
    }
    rho[(uint64_t)c * nq + q] = r;
  }
}

__global__ void k_f64_to_f32_mats(const double *__restrict__ s, float *__restrict__ d, uint64_t n) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    d[t] = (float)s[t];
}

}  // namespace

extern "C" {

int gbfe_op_assemble_local(gbfe_op *op, uint32_t nq, const double *basis_values, const double *weights,
                           const double *fixed_mats, double alpha) {
  if (!op || !basis_values || !weights || nq == 0) return GBFE_ERR_ARG;
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(op->kind == OP_CELL && !op->mat_off_own.p, "assemble_local: needs a per-cell matrix operator");
    GBFE_REQUIRE(me->nd_min == me->nd_max, "assemble_local: cells must all have the same number of dofs");
    const uint32_t nd = me->nd_max;
    DBuf<double> B, w, F;
    B.upload(basis_values, (size_t)nq * nd, ctx->stream);
    w.upload(weights, (size_t)me->n_cells * nq, ctx->stream);
    if (fixed_mats) F.upload(fixed_mats, me->total_mat, ctx->stream);
    k_assemble_local<<<me->n_cells, 256, nq * sizeof(double), ctx->stream>>>(
        B.p, nq, nd, w.p, fixed_mats ? F.p : nullptr, alpha, me->mat_off.p, op->mats.p);
    check_launch(ctx, "assemble_local");
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
  });
}

int gbfe_density(const gbfe_mv *Psi, const double *occupation, uint32_t nq, const double *basis_values,
                 double *rho_host) {
  if (!Psi || !occupation || !basis_values || !rho_host || nq == 0) return GBFE_ERR_ARG;
  gbfe_mesh *me = Psi->mesh;
  gbfe_ctx *ctx = me->ctx;
  return gbfe_guard(ctx, [&] {
    GBFE_REQUIRE(Psi->dtype == GBFE_F64, "density: Psi must be FP64");
    GBFE_REQUIRE(me->nd_min == me->nd_max, "density: cells must all have the same number of dofs");
    const uint32_t nd = me->nd_max, m = Psi->m;
    const size_t smem = sizeof(double) * (size_t)nd * m;
    GBFE_REQUIRE(smem <= 200 * 1024, "density: nd x m too large for one cell tile");
    GBFE_CUDA(cudaFuncSetAttribute(k_density, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DBuf<double> B, occ, rho;
    B.upload(basis_values, (size_t)nq * nd, ctx->stream);
    occ.upload(occupation, m, ctx->stream);
    rho.alloc((size_t)me->n_cells * nq);
    k_density<<<me->n_cells, 128, smem, ctx->stream>>>(Psi->d.p, m, me->ids.p, me->cell_off.p, B.p, nq, occ.p,
                                                       rho.p);
    check_launch(ctx, "density");
    GBFE_CUDA(cudaMemcpyAsync(rho_host, rho.p, (size_t)me->n_cells * nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
    GBFE_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

}  // extern "C"
