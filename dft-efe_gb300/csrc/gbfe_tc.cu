// gbfe_tc.cu -- split-BF16 tensor-core (tcgen05) cell product for the mixed
// precision filter.
//
// Per cell c and vector tile v0..v0+N-1 the kernel computes
//     Yc[j][v] = sum_k A_c(k, j) X[ids_c[k]][v]          (j, k < nd_c)
// i.e. D[M=j][N=v] = A_op[M][K] * B_op[K][N] with A_op[j][k] = A_c(k, j) (the
// column-major cell matrix read row by row) and B_op = the gathered X tile.
// Both operands are split into bf16 pairs (x = hi + lo) and three products
// hi*hi + hi*lo + lo*hi accumulate in FP32 in tensor memory (TMEM).
//
// Data movement:
//   * A hi/lo are pre-split at upload and stored in HBM in the canonical
//     no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core
//     matrix), one contiguous block per (cell, K chunk), so a single 1-D bulk
//     TMA copy (cp.async.bulk) lands a ready tile in shared memory;
//   * X rows are gathered by the CTA's threads (indirect rows: ids_c), split to
//     bf16 hi/lo and written into the same canonical layout (16-byte stores);
//   * tcgen05.mma (cta_group::1, kind::f16, M=128, N=16..256, K=16) is issued
//     by one thread per K step; tcgen05.commit signals an mbarrier when the
//     stage can be refilled; a 3-stage ring overlaps gather/TMA with MMA;
//   * the epilogue reads TMEM with tcgen05.ld (32 lanes x 32 bit per warp) and
//     writes the FP32 cell-wise result, which the deterministic assembly kernel
//     then sums per dof.
// Every mbarrier wait is bounded; on timeout the kernel records an error code
// in a device status word, skips the rest of its work, frees its TMEM and
// returns.
#include "gbfe_internal.cuh"

#include <algorithm>

using namespace gbfe;

namespace gbfe {
void assemble_f32(const gbfe_op *op, const float *Yc, gbfe_mv *Y);
}

namespace {

constexpr int KC = 32;       // K extent of one pipeline stage (2 MMA K-steps)
constexpr int STAGES = 3;
constexpr int THREADS = 128;  // 4 warps: gather, epilogue; thread 0 issues TMA + MMA
constexpr uint32_t CORE_BYTES = 128;             // one 8 x 16-byte core matrix
constexpr uint32_t SBO = (KC / 8) * CORE_BYTES;  // stride between 8-row groups
constexpr uint32_t LBO = CORE_BYTES;             // stride between K-adjacent core matrices
constexpr uint32_t WAIT_LIMIT = 1u << 24;        // bounded mbarrier polls

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((LBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((SBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; no swizzle, base offset 0
  return d;
}

// kind::f16 instruction descriptor: D f32, A bf16, B bf16, both K-major
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bounded wait on the given phase parity; false (and an error code) on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *status, int code) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  atomicCAS(status, 0, code);
  return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// Pre-split A_op = A_c^T into the per-(cell, K chunk) tile layout:
// [hi: MT8 rows x KC][lo: MT8 rows x KC], element (r, kk) at
// (r/8)*(KC/8)*64 + (kk/8)*64 + (r%8)*8 + kk%8.
__global__ void k_build_tc_mats(const double *__restrict__ mats, const uint64_t *__restrict__ mat_off,
                                const uint32_t *__restrict__ cell_off, const uint64_t *__restrict__ a_off,
                                uint32_t n_cells, __nv_bfloat16 *__restrict__ out) {
  const uint32_t c = blockIdx.x;
  if (c >= n_cells) return;
  const uint32_t nd = cell_off[c + 1] - cell_off[c];
  const uint32_t mt8 = (nd + 7) / 8 * 8;
  const uint32_t nk = (nd + KC - 1) / KC;
  const double *A = mats + mat_off[c];
  __nv_bfloat16 *dst = out + a_off[c];
  const uint32_t per_chunk = mt8 * KC;  // elements of one part (hi or lo)
  for (uint32_t idx = threadIdx.x; idx < nk * per_chunk; idx += blockDim.x) {
    const uint32_t kc = idx / per_chunk, rem = idx - kc * per_chunk;
    const uint32_t r = rem / KC, kk = rem - r * KC;
    const uint32_t k = kc * KC + kk;
    const double val = (r < nd && k < nd) ? A[k + (uint64_t)nd * r] : 0.0;
    const __nv_bfloat16 hi = __double2bfloat16(val);
    const __nv_bfloat16 lo = __double2bfloat16(val - (double)__bfloat162float(hi));
    const uint32_t pos = (r / 8) * (KC / 8) * 64 + (kk / 8) * 64 + (r % 8) * 8 + (kk % 8);
    __nv_bfloat16 *base = dst + (uint64_t)kc * 2 * per_chunk;
    base[pos] = hi;
    base[per_chunk + pos] = lo;
  }
}

struct TcShape {
  uint32_t N;       // vector tile (multiple of 16, <= 256)
  uint32_t mtiles;  // 128-row M tiles
  uint32_t a_stage_part;  // bytes of one A part (hi or lo) per stage in smem
  uint32_t b_stage_part;
  uint32_t smem_bytes;
  uint32_t tmem_cols;
};

__host__ TcShape tc_shape(uint32_t N, uint32_t mtiles) {
  TcShape s;
  s.N = N;
  s.mtiles = mtiles;
  s.a_stage_part = mtiles * 128 * KC * 2;
  s.b_stage_part = N * KC * 2;
  s.smem_bytes = STAGES * (2 * s.a_stage_part + 2 * s.b_stage_part) + 1024 /* align */ + 256 /* barriers */;
  uint32_t cols = 32;
  while (cols < mtiles * N) cols *= 2;
  s.tmem_cols = cols;
  return s;
}

__global__ void __launch_bounds__(THREADS, 1) k_cell_apply_tc(
    const float *__restrict__ X, uint32_t m, const uint32_t *__restrict__ ids, const uint32_t *__restrict__ cell_off,
    const uint32_t *__restrict__ bin_cells, const uint64_t *__restrict__ a_off, const __nv_bfloat16 *__restrict__ Atc,
    float *__restrict__ Yc, uint32_t N, uint32_t mtiles, uint32_t tmem_cols, int *__restrict__ status) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t a_part = mtiles * 128 * KC * 2, b_part = N * KC * 2;
  const uint32_t stage_bytes = 2 * a_part + 2 * b_part;
  uint64_t *bars = (uint64_t *)(smem + STAGES * stage_bytes);
  uint64_t *full = bars;                // [STAGES] TMA of A landed
  uint64_t *empty = bars + STAGES;      // [STAGES] MMAs reading the stage done
  uint64_t *done = bars + 2 * STAGES;   // all MMAs done
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 1);

  const uint32_t tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const uint32_t c = bin_cells[blockIdx.x];
  const uint32_t v0 = blockIdx.y * N;
  const uint32_t off = cell_off[c];
  const uint32_t nd = cell_off[c + 1] - off;
  const uint32_t mt8 = (nd + 7) / 8 * 8;
  const uint32_t nk = (nd + KC - 1) / KC;
  const __nv_bfloat16 *Acell = Atc + a_off[c];

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = instr_desc(128, (int)N);
  bool ok = true;

  for (uint32_t kc = 0; kc < nk && ok; ++kc) {
    const uint32_t s = kc % STAGES;
    uint8_t *Ahi = smem + s * stage_bytes;
    uint8_t *Alo = Ahi + a_part;
    uint8_t *Bhi = Alo + a_part;
    uint8_t *Blo = Bhi + b_part;
    if (kc >= STAGES) ok = mbar_wait(&empty[s], ((kc / STAGES) - 1) & 1, status, 1);
    ok = __syncthreads_and(ok ? 1 : 0);  // every thread takes the same branch
    if (!ok) break;
    if (tid == 0) {
      const uint32_t part = mt8 * KC * 2;  // bytes of hi (or lo) for this cell and chunk
      const __nv_bfloat16 *src = Acell + (uint64_t)kc * 2 * mt8 * KC;
      mbar_arrive_expect_tx(&full[s], 2 * part);
      bulk_g2s(Ahi, src, part, &full[s]);
      bulk_g2s(Alo, src + (uint64_t)mt8 * KC, part, &full[s]);
    }
    // gather the X tile: warp-item = (8-dof K block, 32-vector group)
    const uint32_t nvg = N / 32 + ((N % 32) ? 1 : 0);
    for (uint32_t item = warp; item < (KC / 8) * nvg; item += THREADS / 32) {
      const uint32_t kb = item % (KC / 8), vg = item / (KC / 8);
      const uint32_t v = vg * 32 + lane;
      if (v >= N) continue;
      const bool vin = (v0 + v) < m;
      __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const uint32_t k = kc * KC + kb * 8 + kk;
        float x = 0.f;
        if (k < nd && vin) x = X[(uint64_t)ids[off + k] * m + v0 + v];
        split_bf16(x, hi[kk], lo[kk]);
      }
      const uint32_t pos = (v / 8) * SBO + kb * LBO + (v % 8) * 16;
      *(uint4 *)(Bhi + pos) = *(const uint4 *)hi;
      *(uint4 *)(Blo + pos) = *(const uint4 *)lo;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      ok = mbar_wait(&full[s], (kc / STAGES) & 1, status, 2);
      if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t ahi = smem_u32(Ahi), alo = smem_u32(Alo), bhi = smem_u32(Bhi), blo = smem_u32(Blo);
#pragma unroll
        for (uint32_t ks = 0; ks < KC / 16; ++ks) {
          const uint64_t bdh = smem_desc(bhi + ks * 2 * LBO), bdl = smem_desc(blo + ks * 2 * LBO);
          for (uint32_t t = 0; t < mtiles; ++t) {
            const uint32_t aoff = t * 16 * SBO + ks * 2 * LBO;
            const uint64_t adh = smem_desc(ahi + aoff), adl = smem_desc(alo + aoff);
            const uint32_t d = tmem + t * N;
            umma(d, adh, bdh, idesc, (kc | ks) != 0);
            umma(d, adh, bdl, idesc, 1);
            umma(d, adl, bdh, idesc, 1);
          }
        }
        umma_commit(&empty[s]);
      }
    }
    // all threads learn whether thread 0 saw a timeout
    ok = __syncthreads_and(ok ? 1 : 0);
  }
  if (tid == 0 && ok) umma_commit(done);
  if (ok) ok = mbar_wait(done, 0, status, 3);
  ok = __syncthreads_and(ok ? 1 : 0);  // tcgen05.ld below is warp-collective
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue: warp w owns TMEM lanes 32w..32w+31 (rows)
  if (ok) {
    for (uint32_t t = 0; t < mtiles; ++t) {
      const uint32_t row = t * 128 + warp * 32 + lane;
      for (uint32_t col = 0; col < N; col += 16) {
        float v[16];
        tmem_ld16(tmem + ((warp * 32) << 16) + t * N + col, v);
        if (row < nd) {
          float *dst = Yc + (uint64_t)(off + row) * m + v0 + col;
          const uint32_t nvalid = min(16u, m - min(m, v0 + col));
          if (nvalid == 16 && ((((uintptr_t)dst) & 15) == 0)) {
#pragma unroll
            for (int q = 0; q < 4; ++q) ((float4 *)dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          } else {
            for (uint32_t q = 0; q < nvalid; ++q) dst[q] = v[q];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols) : "memory");
  }
}

}  // namespace

namespace gbfe {

// Layout the split-BF16 tiles for every cell (all bins).
void build_tc_mats(gbfe_op *op) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  std::vector<uint64_t> aoff(me->n_cells + 1, 0);
  for (uint32_t c = 0; c < me->n_cells; ++c) {
    const uint64_t nd = me->h_nd[c];
    const uint64_t mt8 = (nd + 7) / 8 * 8, nk = (nd + KC - 1) / KC;
    aoff[c + 1] = aoff[c] + nk * 2 * mt8 * KC;
  }
  op->tc_aoff.upload(aoff.data(), aoff.size(), ctx->stream);
  op->mats_hi.alloc(aoff.back());
  k_build_tc_mats<<<me->n_cells, 256, 0, ctx->stream>>>(op->mats.p, me->mat_off.p, me->cell_off.p, op->tc_aoff.p,
                                                        me->n_cells, op->mats_hi.p);
  check_launch(ctx, "build_tc_mats");
}

bool tc_supported(const gbfe_mesh *me) { return me->nd_max <= 256; }

// Yc (FP32 cell-wise buffer) = split-BF16 tensor-core products, size-binned by
// the number of 128-row M tiles a cell needs.
void cell_apply_tc(const gbfe_op *op, const gbfe_mv *X, float *Yc) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  const uint32_t m = X->m;
  // group bins (distinct nd) into launches by M-tile count
  for (uint32_t mtiles = 1; mtiles <= 2; ++mtiles) {
    uint32_t b0 = UINT32_MAX, b1 = 0;
    for (uint32_t b = 0; b < me->bin_nd.size(); ++b) {
      const uint32_t mt = (me->bin_nd[b] + 127) / 128;
      if (mt == mtiles) {
        b0 = std::min(b0, b);
        b1 = b + 1;
      }
    }
    if (b0 == UINT32_MAX) continue;
    // bins are sorted by nd, so the cells of [b0, b1) are contiguous in bin_cells
    const uint32_t cbeg = me->bin_begin[b0], cend = me->bin_begin[b1];
    const uint32_t ncell = cend - cbeg;
    uint32_t N = std::min<uint32_t>(256, (m + 15) / 16 * 16);
    const uint32_t vt = (m + N - 1) / N;
    N = ((m + vt - 1) / vt + 15) / 16 * 16;  // balance the vector tiles
    const TcShape sh = tc_shape(N, mtiles);
    GBFE_REQUIRE(sh.smem_bytes <= 227 * 1024, "tensor-core tile does not fit in shared memory");
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem_bytes));
    dim3 grid(ncell, vt);
    ProfScope prof(ctx, "cell_apply_mixed", 2.0 * m * (double)me->total_mat * ncell / me->n_cells,
                   4.0 * (2.0 * (double)me->n_dofs * m + (double)me->total_mat) * ncell / me->n_cells);
    k_cell_apply_tc<<<grid, THREADS, sh.smem_bytes, ctx->stream>>>(X->f.p, m, me->ids.p, me->cell_off.p,
                                                                   me->bin_cells.p + cbeg, op->tc_aoff.p,
                                                                   op->mats_hi.p, Yc, N, mtiles, sh.tmem_cols,
                                                                   ctx->status.p);
    check_launch(ctx, "cell_apply_tc");
  }
}

}  // namespace gbfe
