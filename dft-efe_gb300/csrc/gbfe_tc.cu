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
#include "gbfe_tc_ptx.cuh"

#include <algorithm>

using namespace gbfe;

namespace gbfe {
void assemble_f32(const gbfe_op *op, float *Yc, gbfe_mv *Y);
}

namespace {

using namespace gbfe::tc;

// Pre-split A_op = A_c^T into the per-(cell, K chunk) tile layout:
// [hi: MT8 rows x KC][lo: MT8 rows x KC], element (r, kk) at
// (r/8)*(KC/8)*64 + (kk/8)*64 + (r%8)*8 + kk%8.
// kscale (optional): A_c(k, j) *= kscale[ids_c[k]] in FP64 before the split,
// i.e. A diag(kscale): a diagonal operator applied to X folded into A
__global__ void k_build_tc_mats(const double *__restrict__ mats, const uint64_t *__restrict__ mat_off,
                                const uint32_t *__restrict__ cell_off, const uint64_t *__restrict__ a_off,
                                uint32_t n_cells, __nv_bfloat16 *__restrict__ out,
                                const uint32_t *__restrict__ ids = nullptr, const double *__restrict__ kscale = nullptr) {
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
    double val = (r < nd && k < nd) ? A[k + (uint64_t)nd * r] : 0.0;
    if (kscale && r < nd && k < nd) val *= kscale[ids[cell_off[c] + k]];
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
  uint32_t issued = 0;  // thread 0: chunks whose copies were issued

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
      ++issued;
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
  if (tid == 0 && !ok) {
    // a wait gave up: the copy of the chunk that failed may still be landing
    drain_copies(full, issued, STAGES);
  }
  if (tid == 0) umma_commit(done);  // also drains the MMAs on the failure path
  if (ok)
    ok = mbar_wait(done, 0, status, 3);
  else if (tid == 0)
    mbar_wait(done, 0, nullptr, 0);
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
#pragma unroll
            for (uint32_t q = 0; q < 16; ++q)
              if (q < nvalid) dst[q] = v[q];
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


// ---------------------------------------------------------------------------
// v2: persistent, warp-specialised, continuous chunk stream across cells.
//   warps 0..GW-1  gather X chunks into the B ring (one mbarrier arrive per
//              warp per chunk) and run the epilogue of the previous cell (TMEM
//              -> Yc; warp w reads the lanes of quadrant w % 4, every
//              (GW / 4)-th block of 16 columns)
//   warp GW    lane 0 issues the bulk TMA copies of A up to `stages` chunks ahead
//   warp GW+1  allocates TMEM; lane 0 issues tcgen05.mma and the commits
// Sixteen gather warps per SM -- two CTAs of 8 (registers capped by the
// launch bounds) or one CTA of 16 -- keep the gather's indirect row loads in
// flight: they are the latency to hide.  TMEM holds `nbuf` accumulator
// buffers so one cell's epilogue overlaps the next cell's MMAs.  The main loop
// synchronises through mbarriers only.
// ---------------------------------------------------------------------------
constexpr int MAX_STAGES = 4;
constexpr int GATHER_WARPS = 8;
constexpr int TMA_WARP2 = GATHER_WARPS, MMA_WARP2 = GATHER_WARPS + 1;
constexpr int THREADS2 = (GATHER_WARPS + 2) * 32;

struct Tc2Args {
  const float *X;
  uint32_t m;
  const uint32_t *ids;
  const uint32_t *cell_off;
  const uint32_t *cells;  // this launch's cells (one size bin group)
  uint32_t ncells;
  uint32_t vt;            // vector tiles per cell
  const uint64_t *a_off;
  const __nv_bfloat16 *Atc;
  float *Yc;
  uint32_t N, mtiles, tmem_cols, nbuf, stages;
  int *status;
  // optional: X rows [sub_begin, sub_begin + sub_n) are taken from xsub (rows
  // of B^-1 X computed beforehand: the dense enrichment block of the inverse
  // overlap; the diagonal part of B^-1 is folded into the tiles)
  const float *xsub;
  uint32_t sub_begin, sub_n;
  // > 0: float4 gather (m % 4 == 0, 16-byte aligned X / xsub): groups of wpc
  // warps (a power of two, wpc * 32 lanes >= (KC / 8) * N / 4) each own every
  // (GATHER_WARPS / wpc)-th chunk; 0: one scalar row element per lane
  uint32_t wpc;
  // float4 gather only: > 0 = the X rows of a group's next pf chunks are
  // copied (cp.async) into lane-private shared staging ahead of use, so loads
  // stay in flight through stage waits and epilogues; 0 = loads into registers
  uint32_t pf;
  uint32_t a_part;  // bytes of one A part (hi or lo) per stage: the group's largest cell, 8-row padded
  // 0: cell rows on M (mtiles x 128), vectors on N; 1 (swapped): the 128
  // vectors of the tile on M, the cell's rows on N (ncol = rows rounded up to
  // 16): one MMA shape per K step whatever the cell size, and the epilogue
  // writes each cell row's 128 vectors as whole 128-byte lines
  uint32_t swap;
  uint32_t ncol;  // TMEM columns of one accumulator buffer
};

// GW gather / epilogue warps (8, or 16 for one CTA per SM).
// MINB: resident CTAs per SM the registers are budgeted for (2: 96 per thread;
// 3: 64, a few spilled) -- more CTAs keep more gather loads in flight
template <int MINB, int GW>
__global__ void __launch_bounds__((GW + 2) * 32, MINB) k_cell_apply_tc2(const Tc2Args a) {
  constexpr int GATHER_WARPS = GW;
  constexpr int TMA_WARP2 = GW, MMA_WARP2 = GW + 1;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t N = a.N, mtiles = a.mtiles, S = a.stages, nbuf = a.nbuf, m = a.m;
  // A parts hold the group's largest cell (a.a_part bytes); the MMAs of the
  // last M tile read up to mtiles * 128 rows, the rows past the cell's own
  // coming from whatever follows (the allocation is padded for the last
  // stage): they only feed accumulator rows >= nd, which are never stored
  const uint32_t a_part = a.a_part, b_part = N * KC * 2;
  const uint32_t stage_bytes = 2 * a_part + 2 * b_part;
  // float4 gather: groups of wpc warps take ring chunks round robin.  A
  // group's parity wait on a stage is only unambiguous when at most S chunks
  // are in flight, so there are never more groups than stages.
  uint32_t wpc = a.wpc;
  if (wpc)
    while (GATHER_WARPS / wpc > S) wpc *= 2;
  const uint32_t P = wpc ? a.pf : 0;
  const uint32_t stg_lanes = (KC / 8) * (N / 4);  // lanes of a group that gather (float4 mode)
  const uint32_t stg_bytes = P ? (GATHER_WARPS / wpc) * (P + 1) * 8 * stg_lanes * 16 : 0;
  const uint32_t pad = (a.swap ? a.ncol : mtiles * 128) * KC * 2 - a_part;  // rows the MMAs read past a_part
  uint64_t *bars = (uint64_t *)(smem + S * stage_bytes + stg_bytes + pad);
  uint64_t *full_a = bars;
  uint64_t *full_b = bars + MAX_STAGES;
  uint64_t *empty = bars + 2 * MAX_STAGES;
  uint64_t *tfull = bars + 3 * MAX_STAGES;
  uint64_t *tempty = tfull + 2;
  uint64_t *spare = tempty + 2;  // drain_mmas before TMEM is freed
  uint32_t *tmem_slot = (uint32_t *)(spare + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

  const uint32_t tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const uint32_t n_items = a.ncells * a.vt;

  if (tid == 0) {
    for (uint32_t s = 0; s < MAX_STAGES; ++s) {
      mbar_init(&full_a[s], 1);
      mbar_init(&full_b[s], wpc ? wpc : GATHER_WARPS);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], GATHER_WARPS);
    }
    mbar_init(spare, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP2) {
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

  if (warp == TMA_WARP2) {
    // ---------------- TMA producer for A
    if (lane == 0) {
      // plain L2 policy: the four vector tiles of a cell read its tiles at
      // about the same time (an evict-first hint cost 2.5 % here)
      uint32_t q = 0;
      for (uint32_t it = blockIdx.x; it < n_items && !*abort_flag; it += gridDim.x) {
        const uint32_t c = a.cells[it / a.vt];
        const uint32_t nd = a.cell_off[c + 1] - a.cell_off[c];
        const uint32_t mt8 = (nd + 7) / 8 * 8, nk = (nd + KC - 1) / KC;
        const __nv_bfloat16 *Acell = a.Atc + a.a_off[c];
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          const uint32_t s = q % S;
          if (q >= S && !wait(&empty[s], ((q / S) - 1) & 1, 11)) break;
          uint8_t *Ahi = smem + s * stage_bytes;
          const uint32_t part = mt8 * KC * 2;
          const __nv_bfloat16 *src = Acell + (uint64_t)kc * 2 * mt8 * KC;
          mbar_arrive_expect_tx(&full_a[s], 2 * part);
          bulk_g2s(Ahi, src, part, &full_a[s]);
          bulk_g2s(Ahi + a_part, src + (uint64_t)mt8 * KC, part, &full_a[s]);
        }
      }
      drain_copies(full_a, q, S);
    }
    __syncwarp();  // lanes 1-31 wait for lane 0 before the CTA barrier
  } else if (warp == MMA_WARP2) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = instr_desc(128, (int)(a.swap ? a.ncol : N));
      uint32_t q = 0, li = 0;
      for (uint32_t it = blockIdx.x; it < n_items && !*abort_flag; it += gridDim.x, ++li) {
        const uint32_t c = a.cells[it / a.vt];
        const uint32_t nd = a.cell_off[c + 1] - a.cell_off[c];
        const uint32_t nk = (nd + KC - 1) / KC;
        const uint32_t b = li % nbuf;
        if (li >= nbuf && !wait(&tempty[b], ((li / nbuf) - 1) & 1, 12)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bool ok = true;
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          const uint32_t s = q % S;
          if (!wait(&full_a[s], (q / S) & 1, 13) || !wait(&full_b[s], (q / S) & 1, 14)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          uint8_t *Ahi = smem + s * stage_bytes;
          const uint32_t ahi = smem_u32(Ahi), alo = ahi + a_part, bhi = alo + a_part, blo = bhi + b_part;
          if (a.swap) {
            // D[v][j] += X[v][k] A_c(k, j): the gathered tile is the M operand
            const uint32_t d = tmem + b * a.ncol;
#pragma unroll
            for (uint32_t ks = 0; ks < KC / 16; ++ks) {
              const uint64_t xdh = smem_desc(bhi + ks * 2 * LBO), xdl = smem_desc(blo + ks * 2 * LBO);
              const uint64_t adh = smem_desc(ahi + ks * 2 * LBO), adl = smem_desc(alo + ks * 2 * LBO);
              umma(d, xdh, adh, idesc, (kc | ks) != 0);
              umma(d, xdl, adh, idesc, 1);
              umma(d, xdh, adl, idesc, 1);
            }
          } else {
#pragma unroll
            for (uint32_t ks = 0; ks < KC / 16; ++ks) {
              const uint64_t bdh = smem_desc(bhi + ks * 2 * LBO), bdl = smem_desc(blo + ks * 2 * LBO);
              for (uint32_t t = 0; t < mtiles; ++t) {
                const uint32_t aoff = t * 16 * SBO + ks * 2 * LBO;
                const uint64_t adh = smem_desc(ahi + aoff), adl = smem_desc(alo + aoff);
                const uint32_t d = tmem + b * a.ncol + t * N;
                umma(d, adh, bdh, idesc, (kc | ks) != 0);
                umma(d, adh, bdl, idesc, 1);
                umma(d, adl, bdh, idesc, 1);
              }
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tfull[b]);
      }
      drain_mmas(spare);
    }
    __syncwarp();
  } else {
    // ---------------- gather warps (0 .. GW-1) + epilogue
    const uint32_t nvg = (N + 31) / 32;
    const uint32_t lag = nbuf - 1;  // with two TMEM buffers the epilogue trails by one cell
    auto epilogue = [&](uint32_t li, uint32_t it) -> bool {
      const uint32_t c = a.cells[it / a.vt];
      const uint32_t v0 = (it % a.vt) * N;
      const uint32_t off = a.cell_off[c], nd = a.cell_off[c + 1] - off;
      const uint32_t b = li % nbuf;
      bool ok = wait(&tfull[b], (li / nbuf) & 1, 15);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) return false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t quad = warp % 4;
      if (a.swap) {
        // TMEM lane = vector of the tile, column = cell row: each store
        // instruction writes 32 consecutive vectors of one row
        const uint32_t v = quad * 32 + lane;
        const bool vok = v0 + v < m;
        for (uint32_t col = (warp / 4) * 16; col < a.ncol; col += 16 * (GATHER_WARPS / 4)) {
          float val[16];
          tmem_ld16(tmem + ((quad * 32) << 16) + b * a.ncol + col, val);
          if (vok) {
            float *dst = a.Yc + (uint64_t)(off + col) * m + v0 + v;
            if (col + 16 <= nd) {
#pragma unroll
              for (uint32_t i = 0; i < 16; ++i, dst += m) *dst = val[i];
            } else {
#pragma unroll
              for (uint32_t i = 0; i < 16; ++i, dst += m)
                if (col + i < nd) *dst = val[i];
            }
          }
        }
      } else
      for (uint32_t t = 0; t < mtiles; ++t) {
        const uint32_t row = t * 128 + quad * 32 + lane;
        for (uint32_t col = (warp / 4) * 16; col < N; col += 16 * (GATHER_WARPS / 4)) {
          float v[16];
          tmem_ld16(tmem + ((quad * 32) << 16) + b * a.ncol + t * N + col, v);
          if (row < nd) {
            float *dst = a.Yc + (uint64_t)(off + row) * m + v0 + col;
            const uint32_t nvalid = min(16u, m - min(m, v0 + col));
            if (nvalid == 16 && ((((uintptr_t)dst) & 15) == 0)) {
#pragma unroll
              for (int qq = 0; qq < 4; ++qq)
                ((float4 *)dst)[qq] = make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
            } else {
#pragma unroll
              for (uint32_t qq = 0; qq < 16; ++qq)
                if (qq < nvalid) dst[qq] = v[qq];
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
      return true;
    };
    uint32_t q = 0, li = 0, prev_it = 0;
    bool ok = true;
    if (wpc) {
      // float4 gather.  Lane-item (kb, vq) of a chunk = 8 rows (kb*8 ..) x 4
      // vectors (4*vq ..): 8 independent 16-byte row loads per lane, split and
      // stored as four 16-byte K-major rows of the B tile.  A group of wpc
      // warps covers one chunk; the G groups take chunks round robin, so G
      // chunks are gathered concurrently.  Without prefetch the loads are
      // issued before the wait for the ring stage; with prefetch (P chunks
      // ahead, cp.async into lane-private staging) they are issued P of the
      // group's chunks earlier and stay in flight through the epilogues.
      const uint32_t G = GATHER_WARPS / wpc, grp = warp / wpc;
      const uint32_t nq = N / 4, L = (warp % wpc) * 32 + lane;
      const uint32_t kb = L / nq, vq = L % nq;
      const bool active = L < stg_lanes;
      uint8_t *stg = smem + S * stage_bytes + grp * (P + 1) * 8 * stg_lanes * 16 + L * 16;
      // prefetch cursor: the group's chunks in the order the loop below takes them
      uint32_t p_it = blockIdx.x, p_kc = 0, p_q = 0, p_nk = 0, p_off = 0, p_nd = 0, p_v0 = 0;
      auto p_load = [&]() {
        if (p_it < n_items) {
          const uint32_t c = a.cells[p_it / a.vt];
          p_v0 = (p_it % a.vt) * N;
          p_off = a.cell_off[c];
          p_nd = a.cell_off[c + 1] - p_off;
          p_nk = (p_nd + KC - 1) / KC;
        }
      };
      auto p_step = [&]() {
        if (++p_kc >= p_nk) {
          p_kc = 0;
          p_it += gridDim.x;
          p_load();
        }
        ++p_q;
      };
      auto p_issue = [&](uint32_t slot) {  // one copy group per call, empty past the end
        if (active && p_it < n_items) {
          const bool vin = (p_v0 + 4 * vq) < m;
          const uint32_t k0 = p_kc * KC + kb * 8;
          uint8_t *dst = stg + slot * 8 * stg_lanes * 16;
#pragma unroll
          for (int kk = 0; kk < 8; ++kk) {
            const float *src = a.X;
            uint32_t bytes = 0;
            if (vin && k0 + kk < p_nd) {
              const uint32_t id = a.ids[p_off + k0 + kk];
              const uint32_t e = id - a.sub_begin;
              src = ((a.xsub && e < a.sub_n) ? a.xsub + (uint64_t)e * m : a.X + (uint64_t)id * m) + p_v0 + 4 * vq;
              bytes = 16;
            }
            cp_async16(dst + kk * stg_lanes * 16, src, bytes);
          }
        }
        cp_async_commit();
      };
      if (P) {
        p_load();
        while (p_it < n_items && p_q % G != grp) p_step();
        for (uint32_t p = 0; p < P; ++p) {
          p_issue(p);
          do p_step(); while (p_it < n_items && p_q % G != grp);
        }
      }
      uint32_t j = 0;  // the group's chunks consumed
      for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x, ++li) {
        const uint32_t c = a.cells[it / a.vt];
        const uint32_t v0 = (it % a.vt) * N;
        const uint32_t off = a.cell_off[c], nd = a.cell_off[c + 1] - off;
        const uint32_t nk = (nd + KC - 1) / KC;
        const bool vin = active && (v0 + 4 * vq) < m;
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          if (q % G != grp) continue;
          const uint32_t s = q % S;
          const uint32_t k0 = kc * KC + kb * 8;
          float4 xv[8];
          if (P) {
            p_issue((j + P) % (P + 1));
            do p_step(); while (p_it < n_items && p_q % G != grp);
            cp_async_wait(P);  // this chunk's copies (issued P groups ago) landed
            const uint8_t *src = stg + (j % (P + 1)) * 8 * stg_lanes * 16;
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
              xv[kk] = active ? *reinterpret_cast<const float4 *>(src + kk * stg_lanes * 16)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
            ++j;
          } else {
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
              xv[kk] = (vin && k0 + kk < nd)
                           ? __ldg(reinterpret_cast<const float4 *>(a.X + (uint64_t)a.ids[off + k0 + kk] * m + v0 +
                                                                    4 * vq))
                           : make_float4(0.f, 0.f, 0.f, 0.f);
            if (a.xsub && vin) {
#pragma unroll
              for (int kk = 0; kk < 8; ++kk) {
                const uint32_t e = (k0 + kk < nd ? a.ids[off + k0 + kk] : a.sub_begin + a.sub_n) - a.sub_begin;
                if (e < a.sub_n)
                  xv[kk] = __ldg(reinterpret_cast<const float4 *>(a.xsub + (uint64_t)e * m + v0 + 4 * vq));
              }
            }
          }
          if (q >= S) {
            ok = __all_sync(0xffffffffu, wait(&empty[s], ((q / S) - 1) & 1, 16));
            if (!ok) break;
          }
          if (active) {
            uint8_t *Bhi = smem + s * stage_bytes + 2 * a_part;
            uint8_t *Blo = Bhi + b_part;
            // (the four 16-byte stores of a lane hit two bank groups per
            // 8-lane phase; rotating the store order per lane to spread them
            // cost more select instructions than the conflicts cost time)
#pragma unroll
            for (int w = 0; w < 4; ++w) {
              uint32_t ph[4], pl[4];  // bf16 pairs (k0 + 2j, k0 + 2j + 1) of vector 4 vq + w
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) {
                const float4 &x0 = xv[2 * jj], &x1 = xv[2 * jj + 1];
                __nv_bfloat16 h0, l0, h1, l1;
                split_bf16(w == 0 ? x0.x : w == 1 ? x0.y : w == 2 ? x0.z : x0.w, h0, l0);
                split_bf16(w == 0 ? x1.x : w == 1 ? x1.y : w == 2 ? x1.z : x1.w, h1, l1);
                ph[jj] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                pl[jj] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
              }
              const uint32_t v = 4 * vq + w;
              const uint32_t pos = (v / 8) * SBO + kb * LBO + (v % 8) * 16;
              *(uint4 *)(Bhi + pos) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
              *(uint4 *)(Blo + pos) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
            }
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(&full_b[s]);
        }
        if (!ok) break;
        if (lag && li >= 1) ok = epilogue(li - 1, prev_it);
        if (!lag) ok = ok && epilogue(li, it);
        prev_it = it;
      }
      if (ok && lag && li >= 1) epilogue(li - 1, prev_it);
      if (P) cp_async_wait(0);  // no copy may land after the CTA leaves
    } else {
    for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x, ++li) {
      const uint32_t c = a.cells[it / a.vt];
      const uint32_t v0 = (it % a.vt) * N;
      const uint32_t off = a.cell_off[c], nd = a.cell_off[c + 1] - off;
      const uint32_t nk = (nd + KC - 1) / KC;
      for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
        const uint32_t s = q % S;
        if (q >= S) {
          ok = __all_sync(0xffffffffu, wait(&empty[s], ((q / S) - 1) & 1, 16));
          if (!ok) break;
        }
        uint8_t *Bhi = smem + s * stage_bytes + 2 * a_part;
        uint8_t *Blo = Bhi + b_part;
        for (uint32_t item = warp; item < (KC / 8) * nvg; item += 2 * GATHER_WARPS) {
          // two work items per pass keep 16 independent loads in flight per lane
          float xv[2][8];
          uint32_t vv[2];
          bool has[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const uint32_t itm = item + u * GATHER_WARPS;
            has[u] = itm < (KC / 8) * nvg;
            const uint32_t kb = itm % (KC / 8), vg = itm / (KC / 8);
            vv[u] = vg * 32 + lane;
            const bool vin = has[u] && vv[u] < N && (v0 + vv[u]) < m;
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
              const uint32_t k = kc * KC + kb * 8 + kk;
              xv[u][kk] = (vin && k < nd) ? __ldg(a.X + (uint64_t)a.ids[off + k] * m + v0 + vv[u]) : 0.f;
            }
          }
          if (a.xsub) {  // separate pass: keeps the 16 row loads above independent
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const uint32_t itm = item + u * GATHER_WARPS;
              const uint32_t kb = itm % (KC / 8);
              const bool vin = has[u] && vv[u] < N && (v0 + vv[u]) < m;
#pragma unroll
              for (int kk = 0; kk < 8; ++kk) {
                const uint32_t k = kc * KC + kb * 8 + kk;
                const uint32_t e = ((has[u] && k < nd) ? a.ids[off + k] : a.sub_begin + a.sub_n) - a.sub_begin;
                if (e < a.sub_n) xv[u][kk] = vin ? __ldg(a.xsub + (uint64_t)e * m + v0 + vv[u]) : 0.f;
              }
            }
          }
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const uint32_t itm = item + u * GATHER_WARPS;
            if (!has[u] || vv[u] >= N) continue;
            const uint32_t kb = itm % (KC / 8);
            __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) split_bf16(xv[u][kk], hi[kk], lo[kk]);
            const uint32_t pos = (vv[u] / 8) * SBO + kb * LBO + (vv[u] % 8) * 16;
            *(uint4 *)(Bhi + pos) = *(const uint4 *)hi;
            *(uint4 *)(Blo + pos) = *(const uint4 *)lo;
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&full_b[s]);
      }
      if (!ok) break;
      if (lag && li >= 1) ok = epilogue(li - 1, prev_it);
      if (!lag) ok = ok && epilogue(li, it);
      prev_it = it;
    }
    if (ok && lag && li >= 1) epilogue(li - 1, prev_it);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == MMA_WARP2) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
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
  k_build_tc_mats<<<me->n_cells, 256, 0, ctx->stream>>>(op->mats.p, op_mat_off(op), me->cell_off.p, op->tc_aoff.p,
                                                        me->n_cells, op->mats_hi.p);
  check_launch(ctx, "build_tc_mats");
}

// split-BF16 tiles of A diag(kscale) (same layout and offsets as the plain tiles)
void build_tc_mats_folded(const gbfe_op *op, const double *kscale, DBuf<__nv_bfloat16> &out) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  out.alloc(op->mats_hi.n);
  k_build_tc_mats<<<me->n_cells, 256, 0, ctx->stream>>>(op->mats.p, op_mat_off(op), me->cell_off.p, op->tc_aoff.p,
                                                        me->n_cells, out.p, me->ids.p, kscale);
  check_launch(ctx, "build_tc_mats_folded");
}

bool tc_supported(const gbfe_mesh *me) { return me->nd_max <= 256; }

// v2 launch: persistent grid over (cell, vector tile) items of one M-tile group.
// N_req / stages_req = 0: the tuned shape if one exists, else the heuristic.
// Returns the shape the launch used (stages and prefetch depth reduced until
// the shared memory fits; CTAs per SM from shared memory, TMEM and registers).
struct Tc2Used {
  uint32_t per_sm, stages, pf, nbuf;
};
static Tc2Used launch_tc2(gbfe_ctx *ctx, const gbfe_op *op, const gbfe_mv *X, float *Yc, uint32_t cbeg,
                          uint32_t ncell, uint32_t mtiles, double frac, uint32_t nd_max, uint32_t N_req = 0,
                          uint32_t stages_req = 0, const __nv_bfloat16 *tiles = nullptr, const float *xsub = nullptr,
                          uint32_t sub_begin = 0, uint32_t sub_n = 0, uint32_t occ_req = 0,
                          cudaStream_t stream = nullptr, uint32_t nbuf_req = 0, uint32_t pf_req = 0,
                          uint32_t swap_req = 0) {
  gbfe_mesh *me = op->mesh;
  const uint32_t m = X->m;
  if (!stream) stream = ctx->stream;
  if (!N_req) {
    auto it = ctx->tc_tune.find(std::make_tuple(nd_max, mtiles, m));
    if (it != ctx->tc_tune.end()) {
      N_req = it->second.N;
      stages_req = it->second.stages;
      occ_req = it->second.occ;
      nbuf_req = it->second.nbuf;
      pf_req = it->second.pf;
      swap_req = it->second.swap;
    }
  }
  // 1: one CTA per SM with 16 gather warps; 2, 3: CTAs per SM with 8
  const uint32_t occ = occ_req >= 3 ? 3u : occ_req == 1 ? 1u : 2u;
  const uint32_t gw = occ == 1 ? 16u : (uint32_t)GATHER_WARPS;
  const uint32_t swap = swap_req ? 1u : 0u;
  uint32_t N = std::min<uint32_t>(256, (m + 15) / 16 * 16);
  if (N_req) N = std::min<uint32_t>(N, N_req);
  if (swap) N = 128;  // the vector tile is the M extent
  const uint32_t vt = (m + N - 1) / N;
  if (!swap) N = ((m + vt - 1) / vt + 15) / 16 * 16;
  // A parts sized for the group's largest cell; the rows the MMAs read past
  // it (up to the M tiles, or to the 16-rounded N extent when swapped) stay
  // inside the allocation (pad)
  const uint32_t a_part = (nd_max + 7) / 8 * 8 * KC * 2, b_part = N * KC * 2;
  const uint32_t ncol16 = (nd_max + 15) / 16 * 16;
  GBFE_REQUIRE(a_part <= mtiles * 128 * KC * 2 && ncol16 <= 256, "tensor-core launch: cell larger than its M tiles");
  const uint32_t pad = (swap ? ncol16 : mtiles * 128) * KC * 2 - a_part;
  const uint32_t stage_bytes = 2 * a_part + 2 * b_part;
  // float4 gather when every row of X (and of xsub) starts on a 16-byte boundary
  uint32_t wpc = 0;
  if (m % 4 == 0 && ((uintptr_t)X->f.p % 16) == 0 && ((uintptr_t)xsub % 16) == 0 && ctx->tc_gather4) {
    wpc = 1;
    while (wpc * 32 < (KC / 8) * (N / 4)) wpc *= 2;
  }
  uint32_t pf = wpc ? std::min<uint32_t>(pf_req, 3) : 0;
  auto stg_bytes = [&](uint32_t st, uint32_t p) -> uint32_t {
    if (!p) return 0;
    uint32_t w = wpc;
    while (gw / w > st) w *= 2;  // as the kernel: no more gather groups than stages
    return (gw / w) * (p + 1) * 8 * ((KC / 8) * (N / 4)) * 16;
  };
  uint32_t stages = stages_req ? std::min<uint32_t>(stages_req, MAX_STAGES) : MAX_STAGES;
  const uint32_t reserve = 1024 + 512;
  const uint32_t limit = 227 * 1024;
  while (pf > 0 && stages * stage_bytes + stg_bytes(stages, pf) + pad + reserve > limit) --pf;
  while (stages > 2 && stages * stage_bytes + stg_bytes(stages, pf) + pad + reserve > limit) --stages;
  const uint32_t smem = stages * stage_bytes + stg_bytes(stages, pf) + pad + reserve;
  GBFE_REQUIRE(smem <= limit, "tensor-core tile does not fit in shared memory");
  // two TMEM accumulators (the epilogue of one item overlaps the MMAs of the
  // next) where they fit, unless one was asked for (half the columns: room
  // for another CTA on the SM)
  const uint32_t ncol = swap ? ncol16 : mtiles * N;  // TMEM columns of one accumulator
  const uint32_t nbuf = (2 * ncol <= 512 && nbuf_req != 1) ? 2 : 1;
  uint32_t cols = 32;
  while (cols < nbuf * ncol) cols *= 2;
  // CTAs per SM: shared memory (228 KB per SM, 1 KB of it reserved per CTA),
  // TMEM columns and the register budget of the instantiation
  const uint32_t per_sm =
      std::max<uint32_t>(1, std::min<uint32_t>(std::min<uint32_t>((228 * 1024) / (smem + 1024), 512 / cols), occ));
  const uint32_t items = ncell * vt;
  const uint32_t grid = std::min<uint32_t>(items, per_sm * (uint32_t)ctx->sm_count);
  static PerDeviceOnce attr_once;
  attr_once.run(ctx->device, [&] {
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_tc2<2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_tc2<3, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    GBFE_CUDA(cudaFuncSetAttribute(k_cell_apply_tc2<1, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
  });
  Tc2Args args{X->f.p, m, me->ids.p, me->cell_off.p, me->bin_cells.p + cbeg, ncell, vt, op->tc_aoff.p,
               tiles ? tiles : op->mats_hi.p, Yc, N, mtiles, cols, nbuf, stages, ctx->status.p, xsub, sub_begin,
               sub_n, wpc, pf, a_part, swap, ncol};
  ProfScope prof(ctx, "cell_apply_mixed", 2.0 * m * (double)me->total_mat * frac,
                 4.0 * (2.0 * (double)me->n_dofs * m + (double)me->total_mat) * frac);
  if (occ == 1)
    k_cell_apply_tc2<1, 16><<<grid, (16 + 2) * 32, smem, stream>>>(args);
  else if (per_sm >= 3)
    k_cell_apply_tc2<3, 8><<<grid, THREADS2, smem, stream>>>(args);
  else
    k_cell_apply_tc2<2, 8><<<grid, THREADS2, smem, stream>>>(args);
  check_launch(ctx, "cell_apply_tc2");
  return Tc2Used{per_sm, stages, pf, nbuf};
}

// Yc (FP32 cell-wise buffer) = split-BF16 tensor-core products, size-binned by
// the number of 128-row M tiles a cell needs.
// Independent size groups run concurrently (profiling off): one group that
// does not read the substituted rows goes to the side stream, forked at the
// fork event (recorded by the caller before it computed xsub, or here), and
// joins the context stream before the assembly.
void cell_apply_tc(const gbfe_op *op, const gbfe_mv *X, float *Yc, const __nv_bfloat16 *tiles, const float *xsub,
                   uint32_t sub_begin, uint32_t sub_n, bool fork_recorded) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  const uint32_t m = X->m;
  GBFE_REQUIRE((!tiles && !xsub) || ctx->tc_version == 2, "folded tiles need the persistent tensor-core kernel");
  if (ctx->tc_version == 2) {
    struct Group {
      uint32_t cbeg, ncell, mtiles, nd_max;
      bool sub;
    };
    std::vector<Group> groups;
    for (uint32_t mtiles = 1; mtiles <= 2; ++mtiles) {
      uint32_t b0 = UINT32_MAX, b1 = 0;
      for (uint32_t b = 0; b < me->bin_nd.size(); ++b)
        if ((me->bin_nd[b] + 127) / 128 == mtiles) {
          b0 = std::min(b0, b);
          b1 = b + 1;
        }
      if (b0 == UINT32_MAX) continue;
      // substitution only where the group's cells hold substituted rows
      uint32_t max_id = 0;
      for (uint32_t b = b0; b < b1; ++b) max_id = std::max(max_id, me->bin_max_id[b]);
      groups.push_back(Group{me->bin_begin[b0], me->bin_begin[b1] - me->bin_begin[b0], mtiles, me->bin_nd[b1 - 1],
                             xsub && max_id >= sub_begin});
    }
    int side = -1;
    if (ctx->split_groups && !ctx->profiling && groups.size() >= 2)
      for (size_t g = 0; g < groups.size() && side < 0; ++g)
        if (!groups[g].sub) side = (int)g;
    if (side >= 0) {
      ensure_side_stream(ctx);
      if (!fork_recorded) GBFE_CUDA(cudaEventRecord(ctx->fork_ev, ctx->stream));
      GBFE_CUDA(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev, 0));
    }
    for (size_t g = 0; g < groups.size(); ++g) {
      const Group &G = groups[g];
      launch_tc2(ctx, op, X, Yc, G.cbeg, G.ncell, G.mtiles, (double)G.ncell / me->n_cells, G.nd_max, 0, 0, tiles,
                 G.sub ? xsub : nullptr, sub_begin, G.sub ? sub_n : 0u, 0,
                 (int)g == side ? ctx->side_stream : ctx->stream);
    }
    if (side >= 0) {
      GBFE_CUDA(cudaEventRecord(ctx->join_ev, ctx->side_stream));
      GBFE_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0));
    }
    return;
  }
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

// Time every launch shape of the persistent kernel on this operator with m
// vectors and keep the fastest per launch group.  A group whose shape the
// context already holds (tuned earlier, or loaded from the cache file) is not
// timed again: its line is reported, not added to `fresh`.
void autotune_tc(const gbfe_op *op, uint32_t m, std::vector<std::string> &log, std::vector<std::string> &fresh) {
  gbfe_mesh *me = op->mesh;
  gbfe_ctx *ctx = me->ctx;
  GBFE_REQUIRE(op->tc_aoff.p, "autotune: operator has no tensor-core tiles (build it with GBFE_PREC_MIXED)");
  gbfe_mv X;
  X.mesh = me;
  X.m = m;
  X.dtype = GBFE_F32;
  X.f.alloc(X.count());
  GBFE_CUDA(cudaMemsetAsync(X.f.p, 0, X.count() * 4, ctx->stream));
  DBuf<float> Yc;
  Yc.alloc((size_t)me->total_cell_dofs * m);
  const int was_prof = ctx->profiling;
  ctx->profiling = 0;
  cudaEvent_t e0, e1;
  GBFE_CUDA(cudaEventCreate(&e0));
  GBFE_CUDA(cudaEventCreate(&e1));
  for (uint32_t mtiles = 1; mtiles <= 2; ++mtiles) {
    uint32_t b0 = UINT32_MAX, b1 = 0;
    for (uint32_t b = 0; b < me->bin_nd.size(); ++b)
      if ((me->bin_nd[b] + 127) / 128 == mtiles) {
        b0 = std::min(b0, b);
        b1 = b + 1;
      }
    if (b0 == UINT32_MAX) continue;
    const uint32_t cbeg = me->bin_begin[b0], ncell = me->bin_begin[b1] - cbeg;
    const uint32_t nd_max = me->bin_nd[b1 - 1];
    auto line_of = [&](const TcTune &t) {
      return "tc2 " + std::to_string(nd_max) + " " + std::to_string(mtiles) + " " + std::to_string(m) + " " +
             std::to_string(t.N) + " " + std::to_string(t.stages) + " " + std::to_string(t.occ) + " " +
             std::to_string(t.ms) + " " + std::to_string(t.nbuf) + " " + std::to_string(t.pf) + " " +
             std::to_string(t.swap);
    };
    const auto known = ctx->tc_tune.find(std::make_tuple(nd_max, mtiles, m));
    if (known != ctx->tc_tune.end()) {
      log.push_back(line_of(known->second));
      continue;
    }
    TcTune best;
    best.ms = 1e30f;
    for (uint32_t sw : {0u, 1u})
    for (uint32_t N : {16u, 32u, 64u, 128u, 256u}) {
      if (sw ? N != 128 : (N > std::max<uint32_t>(16, (m + 15) / 16 * 16) && N != 16)) continue;
      for (uint32_t st : {2u, 3u, 4u})
      for (uint32_t occ : {1u, 2u, 3u})
      for (uint32_t nb : {0u, 1u})
      for (uint32_t pf : {0u, 1u, 2u, 3u}) {
        // warm; a shape that cannot hold 3 CTAs per SM runs as the 2-CTA one,
        // one whose stages or prefetch were cut to fit, or that has room for
        // one TMEM buffer only, as another shape: not timed twice
        const Tc2Used used = launch_tc2(ctx, op, &X, Yc.p, cbeg, ncell, mtiles, 0.0, nd_max, N, st, nullptr,
                                        nullptr, 0, 0, occ, ctx->stream, nb, pf, sw);
        if ((occ > 2 && used.per_sm < occ) || used.stages != st || used.pf != pf || (nb == 0 && used.nbuf == 1))
          continue;
        GBFE_CUDA(cudaEventRecord(e0, ctx->stream));
        for (int r = 0; r < 3; ++r)
          launch_tc2(ctx, op, &X, Yc.p, cbeg, ncell, mtiles, 0.0, nd_max, N, st, nullptr, nullptr, 0, 0, occ,
                     ctx->stream, nb, pf, sw);
        GBFE_CUDA(cudaEventRecord(e1, ctx->stream));
        GBFE_CUDA(cudaEventSynchronize(e1));
        int st_word = 0;
        GBFE_CUDA(cudaMemcpy(&st_word, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (st_word)
          throw Error(GBFE_ERR_TIMEOUT, "autotune: a bounded wait gave up (code " + std::to_string(st_word) +
                                            ") at vector tile " + std::to_string(N) + ", " + std::to_string(st) +
                                            " stages");
        float ms = 0.f;
        GBFE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= 3.f;
        if (ms < best.ms) {
          best.ms = ms;
          best.N = N;
          best.stages = st;
          best.occ = occ;
          best.nbuf = nb;
          best.pf = pf;
          best.swap = sw;
        }
      }
    }
    ctx->tc_tune[std::make_tuple(nd_max, mtiles, m)] = best;
    log.push_back(line_of(best));
    fresh.push_back(log.back());
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->profiling = was_prof;
}

}  // namespace gbfe
