// gbfe_mixed.cu -- FP32 cellwise apply for the mixed-precision Chebyshev filter.
//
// Block vectors are FP32 [N][m].  The cell product runs on the tensor cores
// (gbfe_tc.cu, split-BF16, cells of up to 256 dofs) or, when that path is
// switched off or a cell is larger, as an FP32 SIMT product over an FP32 copy
// of the cell matrices.  Assembly and constraints are the same deterministic
// kernels as the FP64 path.
#include "gbfe_internal.cuh"

#include <algorithm>

using namespace gbfe;

namespace gbfe {
void assemble_f32(const gbfe_op *op, float *Yc, gbfe_mv *Y);
}

namespace {

__global__ void k_f64_to_f32(const double *__restrict__ s, float *__restrict__ d, uint64_t n) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    d[t] = (float)s[t];
}

// grid = (cells, vector tiles, row splits); block = 256; smem Xs[nd][mtc]
__global__ void __launch_bounds__(256) k_cell_apply_f32(
    const float *__restrict__ X, uint32_t m, const uint32_t *__restrict__ ids, const uint32_t *__restrict__ cell_off,
    const uint64_t *__restrict__ mat_off, const float *__restrict__ mats, float *__restrict__ Yc, uint32_t mt,
    uint32_t jsplit) {
  extern __shared__ float Xf[];
  const uint32_t c = blockIdx.x;
  const uint32_t v0 = blockIdx.y * mt;
  const uint32_t mtc = min(mt, m - v0);
  const uint32_t off = cell_off[c];
  const uint32_t nd = cell_off[c + 1] - off;
  const float *__restrict__ A = mats + mat_off[c];
  const uint32_t nin = nd * mtc;
  for (uint32_t idx = threadIdx.x; idx < nin; idx += blockDim.x) {
    const uint32_t k = idx / mtc, v = idx - k * mtc;
    Xf[idx] = X[(uint64_t)ids[off + k] * m + v0 + v];
  }
  __syncthreads();
  const uint32_t jper = (nd + jsplit - 1) / jsplit;
  const uint32_t j0 = blockIdx.z * jper;
  const uint32_t j1 = min(nd, j0 + jper);
  if (j0 >= j1) return;
  const uint32_t nout = (j1 - j0) * mtc;
  for (uint32_t o = threadIdx.x; o < nout; o += blockDim.x) {
    const uint32_t jj = o / mtc, v = o - jj * mtc;
    const uint32_t j = j0 + jj;
    const float *__restrict__ Aj = A + (uint64_t)nd * j;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    uint32_t k = 0;
    for (; k + 3 < nd; k += 4) {
      a0 = fmaf(__ldg(Aj + k), Xf[k * mtc + v], a0);
      a1 = fmaf(__ldg(Aj + k + 1), Xf[(k + 1) * mtc + v], a1);
      a2 = fmaf(__ldg(Aj + k + 2), Xf[(k + 2) * mtc + v], a2);
      a3 = fmaf(__ldg(Aj + k + 3), Xf[(k + 3) * mtc + v], a3);
    }
    for (; k < nd; ++k) a0 = fmaf(__ldg(Aj + k), Xf[k * mtc + v], a0);
    Yc[(uint64_t)(off + j) * m + v0 + v] = (a0 + a1) + (a2 + a3);
  }
}

}  // namespace

namespace gbfe {

void build_mixed_mats(gbfe_op *op) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  DBuf<float> *m32 = &op->mats_f32;  // FP32 copy kept beside the FP64 matrices
  const uint64_t n = op->mats_count;
  m32->alloc(n);
  unsigned g = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_f64_to_f32<<<g ? g : 1, 256, 0, ctx->stream>>>(op->mats.p, m32->p, n);
  check_launch(ctx, "f64_to_f32");
  if (tc_supported(me)) build_tc_mats(op);
}

void apply_cell_mixed(const gbfe_op *op, gbfe_mv *X, gbfe_mv *Y) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  GBFE_REQUIRE(op->prec & GBFE_PREC_MIXED, "FP32 apply: operator was not built with GBFE_PREC_MIXED");
  const uint32_t m = X->m;
  op->cellbuf_f32.ensure((size_t)me->total_cell_dofs * m);
  if (ctx->use_tc && op->tc_aoff.p) {
    cell_apply_tc(op, X, op->cellbuf_f32.p);
    assemble_f32(op, op->cellbuf_f32.p, Y);
    return;
  }
  const size_t smem_cap = 96 * 1024;
  uint32_t mt = (uint32_t)std::min<size_t>(m, smem_cap / (sizeof(float) * me->nd_max));
  GBFE_REQUIRE(mt > 0, "cell too large for the FP32 apply");
  const uint32_t vt = (m + mt - 1) / mt;
  mt = (m + vt - 1) / vt;
  uint64_t base = (uint64_t)me->n_cells * vt;
  uint32_t jsplit = 1;
  const uint64_t target = (uint64_t)ctx->sm_count * 12;
  while (base * jsplit < target && jsplit * 8 < me->nd_min) jsplit *= 2;
  static PerDeviceOnce attr_once;
  attr_once.run(ctx->device, [&] {
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cap));
  });
  const size_t smem = sizeof(float) * (size_t)me->nd_max * mt;
  dim3 grid(me->n_cells, vt, jsplit);
  const DBuf<float> *m32 = &op->mats_f32;
  ProfScope prof(ctx, "cell_apply_mixed", 2.0 * m * (double)me->total_mat,
                 4.0 * (2.0 * (double)me->n_dofs * m + (double)me->total_mat));
  k_cell_apply_f32<<<grid, 256, smem, ctx->stream>>>(X->f.p, m, me->ids.p, me->cell_off.p, op_mat_off(op), m32->p,
                                                     op->cellbuf_f32.p, mt, jsplit);
  check_launch(ctx, "cell_apply_f32");
  assemble_f32(op, op->cellbuf_f32.p, Y);
}

}  // namespace gbfe
