// gbfe_ozaki.cu -- FP64-accurate cell product on the BF16 tensor cores
// (the splitting scheme of Ozaki, Ogita, Oishi & Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication", Numer. Algorithms 59, 2012).
//
// GB300 runs FP64 FMA at ~1.25 TFLOP/s, so the FP64 cell product of the plain
// path is bound by the FP64 pipe.  Here each operand is cut into eight
// balanced base-128 digit slices (gbfe_oz.cuh), which BF16 represents exactly:
//     A_op[j][k] = 2^(ea_j+1) sum_s a_s[j][k] 2^-7s     (per-row exponent ea_j)
//     X[i][v]    = 2^(ex_v+1) sum_t x_t[i][v] 2^-7t     (per-vector exponent ex_v)
// with |digits| <= 64 and a truncation error below 2^-55 of the row / vector
// maximum.  For every level g = s + t (2..9) the tensor cores accumulate
//     L_g[j][v] = sum_{s+t=g} sum_k a_s[j][k] x_t[k][v]
// in its own FP32 TMEM accumulator (8 levels x 64 vectors = all 512 columns).
// A level holds at most 8 digit pairs of products <= 2^12, so for cells of up
// to 256 dofs every partial sum stays below 2^23 and the accumulation is
// exact.  The epilogue forms sum_g L_g 2^-7g as an FP32 double-float
// (error-free TwoSum), converts once to FP64 and applies 2^(ea_j + ex_v + 2).
// Products with s + t > 9 are below 2^-63 and are dropped.  Result: the FP64
// product to ~2^-48 relative per entry (normwise); the 36 digit-pair
// products of a K step are issued as 12 MMAs (N up to 256) over stacked slices.
//
// Data movement follows the persistent split-BF16 kernel: A slices are
// pre-laid-out in HBM (per cell, per K chunk of 32, 8 slices in the canonical
// K-major core-matrix layout) and land by bulk TMA copies; X rows are gathered
// by eight warps that cut each FP64 value into digits with integer
// instructions and also run the epilogue; one thread issues tcgen05.mma, one
// thread the bulk copies.
// Cells with more than 128 dofs are processed as two 128-row work items.
#include "gbfe_internal.cuh"
#include "gbfe_oz.cuh"
#include "gbfe_tc_ptx.cuh"

#include <algorithm>

using namespace gbfe;
using namespace gbfe::tc;

namespace {

constexpr int OZ_S = 8;        // slices per operand
constexpr int OZ_N = 64;       // vectors per work item (8 levels x 64 = 512 TMEM columns)
constexpr int OZ_STAGES = 2;
constexpr int OZ_GW = 8;                       // gather / epilogue warps
constexpr int OZ_TMA_WARP = OZ_GW, OZ_MMA_WARP = OZ_GW + 1;
constexpr int OZ_THREADS = (OZ_GW + 2) * 32;
constexpr uint32_t OZ_A_PART = 128 * KC * 2;  // one slice of a 128-row A chunk (bytes)
constexpr uint32_t OZ_B_PART = OZ_N * KC * 2;  // one slice of a B chunk
constexpr uint32_t OZ_STAGE = OZ_S * (OZ_A_PART + OZ_B_PART);
constexpr uint32_t OZ_EPI = OZ_GW * oz::EPI_SCRATCH_DOUBLES * 8;  // epilogue staging, one 4 KB tile per warp
constexpr uint32_t OZ_SMEM = OZ_STAGES * OZ_STAGE + OZ_EPI + 1024 + 512;
static_assert(OZ_SMEM <= 227 * 1024, "sliced cell product: shared memory");

__device__ __forceinline__ void oz_digits(double v, int e, int *d) { oz::digits(v, e, d); }
__device__ __forceinline__ int oz_exponent(double vmax) { return oz::exponent_of(vmax); }

// A_op = A_c^T slices: per (cell, chunk) [slice][MT8 x KC] canonical tiles,
// and per-row exponents (one per cell dof).
__global__ void k_build_oz_mats(const double *__restrict__ mats, const uint64_t *__restrict__ mat_off,
                                const uint32_t *__restrict__ cell_off, const uint64_t *__restrict__ a_off,
                                uint32_t n_cells, __nv_bfloat16 *__restrict__ out, int *__restrict__ row_exp) {
  const uint32_t c = blockIdx.x;
  if (c >= n_cells) return;
  const uint32_t off = cell_off[c], nd = cell_off[c + 1] - off;
  const uint32_t mt8 = (nd + 7) / 8 * 8, nk = (nd + KC - 1) / KC;
  const double *A = mats + mat_off[c];
  for (uint32_t j = threadIdx.x; j < nd; j += blockDim.x) {
    double mx = 0.0;
    for (uint32_t k = 0; k < nd; ++k) mx = fmax(mx, fabs(A[k + (uint64_t)nd * j]));
    row_exp[off + j] = oz_exponent(mx);
  }
  __syncthreads();
  __nv_bfloat16 *dst = out + a_off[c];
  const uint32_t per_slice = mt8 * KC;
  for (uint32_t idx = threadIdx.x; idx < nk * per_slice; idx += blockDim.x) {
    const uint32_t kc = idx / per_slice, rem = idx - kc * per_slice;
    const uint32_t r = rem / KC, kk = rem - r * KC;
    const uint32_t k = kc * KC + kk;
    int d[OZ_S] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (r < nd && k < nd) oz_digits(A[k + (uint64_t)nd * r], row_exp[off + r], d);
    const uint32_t pos = (r / 8) * (KC / 8) * 64 + (kk / 8) * 64 + (r % 8) * 8 + (kk % 8);
    __nv_bfloat16 *base = dst + (uint64_t)kc * OZ_S * per_slice;
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) base[(uint64_t)s * per_slice + pos] = __int2bfloat16_rn(d[s]);
  }
}

// per-vector exponent of the largest |X[i][v]| (two-stage max of the exponent
// bits, integer instructions; max is order-free)
__global__ void k_colmax_partial(const double *__restrict__ X, uint64_t rows, uint32_t m, int *__restrict__ part) {
  oz::colmax_partial_block(X, X, 1, m, rows, part);
}

__global__ void k_colmax_final(const int *__restrict__ part, uint32_t nb, uint32_t m, int *__restrict__ ex) {
  oz::colmax_final_block(part, nb, m, ex);
}

struct OzArgs {
  const double *X;
  uint32_t m;
  const uint32_t *ids;
  const uint32_t *cell_off;
  const uint32_t *cells;  // cells of this launch
  uint32_t ncells;
  uint32_t mts;           // 128-row items per cell in this launch (1 or 2)
  uint32_t vt;            // vector tiles per cell
  const uint64_t *a_off;
  const __nv_bfloat16 *Aoz;
  const int *row_exp;
  const int *x_exp;
  double *Yc;
  uint32_t tmem_cols;
  int *status;
};

__global__ void __launch_bounds__(OZ_THREADS, 1) k_cell_apply_oz(const OzArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  double *epi_scratch = (double *)(smem + OZ_STAGES * OZ_STAGE);
  uint64_t *bars = (uint64_t *)(smem + OZ_STAGES * OZ_STAGE + OZ_EPI);
  uint64_t *full_a = bars;
  uint64_t *full_b = bars + OZ_STAGES;
  uint64_t *empty = bars + 2 * OZ_STAGES;
  uint64_t *tfull = bars + 3 * OZ_STAGES;
  uint64_t *tempty = tfull + 1;
  uint64_t *spare = tempty + 1;  // drain_mmas before TMEM is freed
  uint32_t *tmem_slot = (uint32_t *)(spare + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const uint32_t tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const uint32_t m = a.m;
  const uint32_t per_cell = a.mts * a.vt;
  const uint32_t n_items = a.ncells * per_cell;

  if (tid == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(&full_a[s], 1);
      mbar_init(&full_b[s], OZ_GW);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, OZ_GW);
    mbar_init(spare, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == OZ_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(a.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  auto wait = [&](uint64_t *bar, uint32_t parity, int code) -> bool {
    if (*abort_flag) return false;
    if (mbar_wait(bar, parity, a.status, code)) return true;
    *abort_flag = 1;
    return false;
  };
  auto decode = [&](uint32_t it, uint32_t &c, uint32_t &mt, uint32_t &v0) {
    c = a.cells[it / per_cell];
    const uint32_t rem = it % per_cell;
    mt = rem / a.vt;
    v0 = (rem % a.vt) * OZ_N;
  };

  if (warp == OZ_TMA_WARP) {
    // ---------------- TMA producer: 8 slice tiles per chunk
    if (lane == 0) {
      uint32_t q = 0;
      const uint64_t pol = l2_evict_first_policy();  // slices are read once per launch
      for (uint32_t it = blockIdx.x; it < n_items && !*abort_flag; it += gridDim.x) {
        uint32_t c, mt, v0;
        decode(it, c, mt, v0);
        const uint32_t nd = a.cell_off[c + 1] - a.cell_off[c];
        const uint32_t mt8 = (nd + 7) / 8 * 8, nk = (nd + KC - 1) / KC;
        const uint32_t rows = min(128u, mt8 - 128 * mt);
        const __nv_bfloat16 *Acell = a.Aoz + a.a_off[c];
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          const uint32_t s = q % OZ_STAGES;
          if (q >= OZ_STAGES && !wait(&empty[s], ((q / OZ_STAGES) - 1) & 1, 21)) break;
          uint8_t *Ast = smem + s * OZ_STAGE;
          const uint32_t bytes = rows * KC * 2;
          mbar_arrive_expect_tx(&full_a[s], OZ_S * bytes);
          for (int sl = 0; sl < OZ_S; ++sl) {
            const __nv_bfloat16 *src = Acell + ((uint64_t)kc * OZ_S + sl) * mt8 * KC + (uint64_t)mt * 128 * KC;
            bulk_g2s_stream(Ast + sl * OZ_A_PART, src, bytes, &full_a[s], pol);
          }
        }
      }
      drain_copies(full_a, q, OZ_STAGES);
    }
    __syncwarp();
  } else if (warp == OZ_MMA_WARP) {
    // ---------------- MMA issuer: 36 products per K step into 8 level accumulators
    if (lane == 0) {
      uint32_t q = 0, li = 0;
      for (uint32_t it = blockIdx.x; it < n_items && !*abort_flag; it += gridDim.x, ++li) {
        uint32_t c, mt, v0;
        decode(it, c, mt, v0);
        const uint32_t nd = a.cell_off[c + 1] - a.cell_off[c];
        const uint32_t nk = (nd + KC - 1) / KC;
        if (li >= 1 && !wait(tempty, (li - 1) & 1, 22)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool ok = true;
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          const uint32_t s = q % OZ_STAGES;
          if (!wait(&full_a[s], (q / OZ_STAGES) & 1, 23) || !wait(&full_b[s], (q / OZ_STAGES) & 1, 24)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t abase = smem_u32(smem + s * OZ_STAGE);
          const uint32_t bbase = abase + OZ_S * OZ_A_PART;
          for (uint32_t ks = 0; ks < KC / 16; ++ks) {
            // slice sl of A against the stacked B slices t0..t1 (one descriptor,
            // N = 64 (t1 - t0 + 1)) into the contiguous levels sl+t0 .. sl+t1:
            // 12 MMAs per K step; the two sl = 1 MMAs start every level
#pragma unroll
            for (int sl = 1; sl <= OZ_S; ++sl) {
#pragma unroll
              for (int t0 = 1; t0 <= OZ_S + 1 - sl; t0 += 4) {
                const int t1 = t0 + 3 < OZ_S + 1 - sl ? t0 + 3 : OZ_S + 1 - sl;
                const uint64_t ad = smem_desc(abase + (sl - 1) * OZ_A_PART + ks * 2 * LBO);
                const uint64_t bd = smem_desc(bbase + (t0 - 1) * OZ_B_PART + ks * 2 * LBO);
                umma(tmem + (sl + t0 - 2) * OZ_N, ad, bd, instr_desc(128, OZ_N * (t1 - t0 + 1)),
                     ((kc | ks) == 0 && sl == 1) ? 0u : 1u);
              }
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(tfull);
      }
      drain_mmas(spare);
    }
    __syncwarp();
  } else {
    // ---------------- gather warps 0-7: X rows -> 8 digit slices; epilogue
    // (KC/8) K blocks x (OZ_N/32) vector groups = 8 items per chunk, one per
    // warp: warp w always gathers K block w % 4 of vector group w / 4.  The
    // row loads of the next chunk (of this item, or the first chunk of the
    // next item, across the epilogue) are issued before the current chunk's
    // digits are cut, so their latency overlaps that work.
    static_assert((KC / 8) * (OZ_N / 32) == OZ_GW, "one gather item per warp");
    const uint32_t kb = warp % (KC / 8), vg = warp / (KC / 8);
    const uint32_t v = vg * 32 + lane;
    auto load_chunk = [&](uint32_t it, uint32_t kc, double (&x)[8]) {
      uint32_t c, mt, v0;
      decode(it, c, mt, v0);
      const uint32_t off = a.cell_off[c], nd = a.cell_off[c + 1] - off;
      const bool vin = (v0 + v) < m;
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const uint32_t k = kc * KC + kb * 8 + kk;
        x[kk] = (vin && k < nd) ? __ldg(a.X + (uint64_t)a.ids[off + k] * m + v0 + v) : 0.0;
      }
    };
    uint32_t q = 0, li = 0;
    bool ok = true;
    double xcur[8], xnxt[8];
    if (blockIdx.x < n_items) load_chunk(blockIdx.x, 0, xcur);
    for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x, ++li) {
      uint32_t c, mt, v0;
      decode(it, c, mt, v0);
      const uint32_t off = a.cell_off[c], nd = a.cell_off[c + 1] - off;
      const uint32_t nk = (nd + KC - 1) / KC;
      const bool vin = (v0 + v) < m;
      const int ex = vin ? a.x_exp[v0 + v] : 0;
      for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
        const uint32_t s = q % OZ_STAGES;
        // prefetch: the next chunk of this item, else the first of the next item
        const bool more = kc + 1 < nk || it + gridDim.x < n_items;
        if (more) load_chunk(kc + 1 < nk ? it : it + gridDim.x, kc + 1 < nk ? kc + 1 : 0, xnxt);
        if (q >= OZ_STAGES) {
          ok = __all_sync(0xffffffffu, wait(&empty[s], ((q / OZ_STAGES) - 1) & 1, 25));
          if (!ok) break;
        }
        uint8_t *Bst = smem + s * OZ_STAGE + OZ_S * OZ_A_PART;
        uint32_t packed[OZ_S][4];
#pragma unroll
        for (int kk = 0; kk < 8; kk += 2) {
          uint32_t pp[OZ_S];
          oz::digits_pair_bf16(xcur[kk], xcur[kk + 1], ex, pp);
#pragma unroll
          for (int sl = 0; sl < OZ_S; ++sl) packed[sl][kk / 2] = pp[sl];
        }
        const uint32_t pos = (v / 8) * SBO + kb * LBO + (v % 8) * 16;
#pragma unroll
        for (int sl = 0; sl < OZ_S; ++sl)
          *(uint4 *)(Bst + sl * OZ_B_PART + pos) = make_uint4(packed[sl][0], packed[sl][1], packed[sl][2], packed[sl][3]);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&full_b[s]);
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) xcur[kk] = xnxt[kk];
      }
      if (!ok) break;
      // epilogue of this item (single TMEM buffer)
      ok = __all_sync(0xffffffffu, wait(tfull, li & 1, 26));
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // warp w reads TMEM lanes of quadrant w % 4, columns [32 (w / 4), +32),
      // 16 at a time, staged through its scratch tile into whole-row stores
      const uint32_t quad = warp % 4, colh = warp / 4;
      const uint32_t row = mt * 128 + quad * 32 + lane;
      const int er = row < nd ? a.row_exp[off + row] : 0;
      double *scr = epi_scratch + warp * oz::EPI_SCRATCH_DOUBLES;
      for (uint32_t col = colh * 32; col < colh * 32 + 32; col += 16) {
        int xe[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) xe[j] = (v0 + col + j < m) ? a.x_exp[v0 + col + j] : 0;
        oz::combine16_to_scratch(tmem + ((quad * 32) << 16) + col, OZ_N, scr, lane, er, xe);
        const uint32_t j = lane % 16, v = v0 + col + j;
#pragma unroll 4
        for (uint32_t i = 0; i < 16; ++i) {
          const uint32_t r = 2 * i + lane / 16, orow = mt * 128 + quad * 32 + r;
          if (orow < nd && v < m) a.Yc[(uint64_t)(off + orow) * m + v] = oz::scratch_at(scr, r, j);
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == OZ_MMA_WARP) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
  }
}

}  // namespace

namespace gbfe {

bool oz_supported(const gbfe_mesh *me) { return me->nd_max <= 256; }

void build_oz_mats(gbfe_op *op) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  std::vector<uint64_t> aoff(me->n_cells + 1, 0);
  for (uint32_t c = 0; c < me->n_cells; ++c) {
    const uint64_t nd = me->h_nd[c];
    const uint64_t mt8 = (nd + 7) / 8 * 8, nk = (nd + KC - 1) / KC;
    aoff[c + 1] = aoff[c] + nk * OZ_S * mt8 * KC;
  }
  op->oz_aoff.upload(aoff.data(), aoff.size(), ctx->stream);
  op->oz_mats.alloc(aoff.back());
  op->oz_row_exp.alloc(me->total_cell_dofs);
  k_build_oz_mats<<<me->n_cells, 128, 0, ctx->stream>>>(op->mats.p, op_mat_off(op), me->cell_off.p, op->oz_aoff.p,
                                                        me->n_cells, op->oz_mats.p, op->oz_row_exp.p);
  check_launch(ctx, "build_oz_mats");
}

// Yc (FP64 cell-wise buffer) = FP64-accurate sliced tensor-core products
// per-column exponents of X into op's buffer (context stream)
const int *oz_column_exponents(const gbfe_op *op, const gbfe_mv *X) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  const uint32_t m = X->m;
  const uint64_t rows = me->n_dofs;
  const unsigned nb = (unsigned)std::min<uint64_t>(8 * (uint64_t)ctx->sm_count, std::max<uint64_t>(1, rows));
  ctx->oz_ipart.ensure((size_t)nb * m);
  op->oz_xexp.ensure(m);
  k_colmax_partial<<<nb, oz::COLMAX_THREADS, 0, ctx->stream>>>(X->d.p, rows, m, ctx->oz_ipart.p);
  k_colmax_final<<<(m + 31) / 32, oz::COLMAX_FINAL_THREADS, 0, ctx->stream>>>(ctx->oz_ipart.p, nb, m,
                                                                             op->oz_xexp.p);
  count_launch(ctx, 2);
  return op->oz_xexp.p;
}

void cell_apply_oz(const gbfe_op *op, const gbfe_mv *X, double *Yc, const int *xexp, cudaStream_t stream) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  const uint32_t m = X->m;
  if (!stream) stream = ctx->stream;
  if (!xexp) xexp = oz_column_exponents(op, X);
  const uint32_t vt = (m + OZ_N - 1) / OZ_N;
  const uint32_t smem = OZ_SMEM;
  static PerDeviceOnce attr_once;
  attr_once.run(ctx->device, [&] {
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  });
  for (uint32_t mts = 1; mts <= 2; ++mts) {
    uint32_t b0 = UINT32_MAX, b1 = 0;
    for (uint32_t b = 0; b < me->bin_nd.size(); ++b)
      if ((me->bin_nd[b] + 127) / 128 == mts) {
        b0 = std::min(b0, b);
        b1 = b + 1;
      }
    if (b0 == UINT32_MAX) continue;
    const uint32_t cbeg = me->bin_begin[b0], ncell = me->bin_begin[b1] - cbeg;
    const uint32_t items = ncell * mts * vt;
    const uint32_t grid = std::min<uint32_t>(items, (uint32_t)ctx->sm_count);
    OzArgs args{X->d.p, m, me->ids.p, me->cell_off.p, me->bin_cells.p + cbeg, ncell, mts, vt, op->oz_aoff.p,
                op->oz_mats.p, op->oz_row_exp.p, xexp, Yc, 512, ctx->status.p};
    const double frac = (double)ncell / me->n_cells;
    ProfScope prof(ctx, "cell_apply_f64_oz", 2.0 * m * (double)me->total_mat * frac,
                   8.0 * (2.0 * (double)me->n_dofs * m + (double)me->total_mat) * frac);
    k_cell_apply_oz<<<grid, OZ_THREADS, smem, stream>>>(args);
    check_launch(ctx, "cell_apply_oz");
  }
}

}  // namespace gbfe
