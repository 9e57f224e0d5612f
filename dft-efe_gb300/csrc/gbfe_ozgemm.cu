// gbfe_ozgemm.cu -- FP64-accurate tall-skinny products of the subspace
// stages on the BF16 tensor cores (sliced as in gbfe_oz.cuh).
//
// The Rayleigh-Ritz / Cholesky-GS stages of a ChFSI pass spend their FP64
// flops in two shapes (ChebyshevFilteredEigenSolver.t.cpp:194-437 through
// OrthonormalizationFunctions.t.cpp:356-415 and
// RayleighRitzEigenSolver.t.cpp:233-301):
//   * Gram matrices  S_o = A_o^T B      (A_o, B: N x m blocks, K = N long)
//   * rotations      out_o = Y_o T     (Y_o: N x m, T: m x m, K = m short)
// GB300's FP64 pipe caps both near 1.1 TFLOP/s.  Here each FP64 operand is
// cut into its 8 digit slices ONCE, by an HBM-bound slicing pass
// (k_oz_slice_cols: per-column exponents, Gram operands; k_oz_slice_rows:
// per-row exponents, rotation inputs) that writes the digits straight in the
// MMA operand layout (canonical K-major tiles, 8 slices of 128 x KC or 64 x KC
// BF16 per K stage).  The product kernels then only move tiles and multiply:
//   k_oz_gram: work item = (128 stacked A columns, 64 columns of B, a range of
//     512-row K chunks).  One warp bulk-copies the A and B digit tiles of each
//     K stage, one thread issues 36 tcgen05.mma per 16-row K step into 8 level
//     accumulators (all 512 TMEM columns); after every 512 rows (the exact
//     FP32 range) eight warps drain TMEM into FP64 registers.  Items are
//     ordered K range first, so the items sharing a K range (and so the same
//     digit tiles) run at the same time and read them from L2; their count is
//     a multiple of the SM count.  Each item writes its partial;
//     k_oz_gram_final sums the partials in a fixed order (deterministic).
//   * k_oz_rot: work item = (operand, 128 rows, 64 output columns); the m x m
//     factor is sliced once per call (k_oz_build_t); the row digit tiles and
//     the factor tiles land by bulk copies; one TMEM pass covers K = m <= 512;
//     eight warps run the epilogue.  An operand may be two row blocks side by
//     side (K = 2m) with its own factor: the residual HY T - MY T diag(eps) of
//     the rotated block is [HY | MY] [T; -T diag(eps)], one product.
// Slicing each value once instead of once per 64-column output tile is what
// keeps the tensor pipe fed at m = 512: the digit cut is ~60 integer
// instructions per value.
// Every wait is bounded (error status, no hang); TMEM is freed on every exit.
#include "gbfe_internal.cuh"
#include "gbfe_oz.cuh"
#include "gbfe_tc_ptx.cuh"

#include <algorithm>
#include <memory>

using namespace gbfe;
using namespace gbfe::tc;

namespace {

constexpr int PW = 8;                      // producer / epilogue warps
constexpr int OG_THREADS = (PW + 2) * 32;  // + TMA warp + MMA warp
constexpr int OG_N = 64;                   // output columns per item (8 levels x 64 = 512 TMEM columns)
constexpr int OG_STAGES = 2;
constexpr uint32_t A_PART = 128 * KC * 2;  // one slice of a 128 x KC tile (bytes)
constexpr uint32_t B_PART = OG_N * KC * 2;
constexpr uint32_t OG_STAGE = oz::S * (A_PART + B_PART);
constexpr uint32_t OG_EPI = PW * oz::EPI_SCRATCH_DOUBLES * 8;  // rotation epilogue staging, 4 KB per warp
constexpr uint32_t OG_SMEM = OG_STAGES * OG_STAGE + OG_EPI + 1024 + 512;
static_assert(OG_SMEM <= 227 * 1024, "sliced dense products: shared memory");
constexpr uint32_t CHUNK = oz::K_EXACT;    // Gram rows per exact TMEM accumulation
constexpr uint32_t STAGES_PER_CHUNK = CHUNK / KC;
constexpr uint32_t TILE = 128 * OG_N;      // elements of one partial tile

// write the 8 slices of 8 consecutive K values (one 16-byte core row each)
__device__ __forceinline__ void store_core_rows(uint8_t *tile, uint32_t part, uint32_t pos, const double *v, int e) {
  uint32_t packed[oz::S][4];
#pragma unroll
  for (int kk = 0; kk < 8; kk += 2) {
    uint32_t pp[oz::S];
    oz::digits_pair_bf16(v[kk], v[kk + 1], e, pp);
#pragma unroll
    for (int s = 0; s < oz::S; ++s) packed[s][kk / 2] = pp[s];
  }
#pragma unroll
  for (int s = 0; s < oz::S; ++s)
    *(uint4 *)(tile + s * part + pos) = make_uint4(packed[s][0], packed[s][1], packed[s][2], packed[s][3]);
}

// 8 consecutive values Y[row][k0 .. k0+8) of a row of the N x K operand made
// of the rows of Y (columns 0 .. m-1) and, for K = 2m, Y2 side by side; zero
// past the ends.  Two 16-byte loads per pair of values when the 8 values lie
// in one block and are 16-byte aligned.
__device__ __forceinline__ void load_row8(const double *__restrict__ Y, const double *__restrict__ Y2, uint32_t m,
                                          uint32_t K, uint64_t row, uint64_t N, uint32_t k0, double *v) {
  if (row >= N) {
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) v[kk] = 0.0;
    return;
  }
  if (k0 + 8 <= K && (k0 + 8 <= m || k0 >= m)) {
    const double *src = k0 < m ? Y + row * m + k0 : Y2 + row * m + (k0 - m);
    if (((uintptr_t)src & 15u) == 0) {
#pragma unroll
      for (int kk = 0; kk < 8; kk += 2) {
        const double2 t = __ldg((const double2 *)(src + kk));
        v[kk] = t.x;
        v[kk + 1] = t.y;
      }
      return;
    }
  }
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const uint32_t k = k0 + kk;
    v[kk] = k < K ? __ldg(k < m ? Y + row * m + k : Y2 + row * m + (k - m)) : 0.0;
  }
}

// Digit tiles of the rows of an N x K operand (see load_row8) with per-row
// exponents rexp: tile (row tile rt, K stage kc) = 8 slices of 128 x KC BF16
// in the canonical K-major layout, tiles in (rt, kc) order, rows past N and K
// values past K zero.  Thread (row r, K group g of 8 values): four threads
// read a row's 256 contiguous bytes; for each slice, the eight rows of a
// warp with the same g write one 128-byte core matrix.
__global__ void __launch_bounds__(256) k_oz_slice_rows(const double *__restrict__ Y, const double *__restrict__ Y2,
                                                       uint32_t m, uint32_t K, uint64_t N,
                                                       const int *__restrict__ rexp, uint32_t kchunks,
                                                       uint64_t ntiles, uint8_t *__restrict__ out) {
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t rt = tile / kchunks;
    const uint32_t kc = (uint32_t)(tile % kchunks);
    uint8_t *dst = out + tile * (oz::S * A_PART);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t r = h * 64 + threadIdx.x / 4, g = threadIdx.x % 4;
      const uint64_t row = rt * 128 + r;
      double v[8];
      load_row8(Y, Y2, m, K, row, N, kc * KC + g * 8, v);
      store_core_rows(dst, A_PART, (r / 8) * SBO + g * LBO + (r % 8) * 16, v, row < N ? rexp[row] : 0);
    }
  }
}

// Digit tiles of the columns of up to two stacked N x ma row-major blocks
// (column c < ma of A0, else column c - ma of A1; cols columns in all) with
// per-column exponents cexp: tile (column tile ct of W columns, K stage kc
// of KC rows) = 8 slices of W x KC BF16, K-major (a core row holds 8
// consecutive rows of one column), tiles in (ct, kc) order, zero past N
// and past cols.  A warp's 32 consecutive columns read 256 contiguous
// bytes per row and write four 128-byte core matrices per slice.
template <int W>
__global__ void __launch_bounds__(256) k_oz_slice_cols(const double *__restrict__ A0, const double *__restrict__ A1,
                                                       uint32_t ma, uint32_t cols, uint64_t N,
                                                       const int *__restrict__ cexp, uint32_t kchunks,
                                                       uint64_t ntiles, uint8_t *__restrict__ out) {
  constexpr uint32_t PART = W * KC * 2;
  static_assert((W * 4) % 256 == 0, "whole passes of 256 threads");
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t ct = (uint32_t)(tile / kchunks), kc = (uint32_t)(tile % kchunks);
    uint8_t *dst = out + tile * (oz::S * PART);
#pragma unroll
    for (int h = 0; h < W * 4 / 256; ++h) {
      const uint32_t p = threadIdx.x + 256 * h, c = p % W, g = p / W;
      const uint32_t col = ct * W + c;
      const bool cin = col < cols;
      const double *src = cin ? (col < ma ? A0 + col : A1 + (col - ma)) : nullptr;
      double v[8];
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const uint64_t k = (uint64_t)kc * KC + g * 8 + kk;
        v[kk] = (cin && k < N) ? __ldg(src + k * ma) : 0.0;
      }
      store_core_rows(dst, PART, (c / 8) * SBO + g * LBO + (c % 8) * 16, v, cin ? cexp[col] : 0);
    }
  }
}

// The 36 digit-pair products of one 16-row K step as 12 MMAs: slice s of A
// against the stacked B slices t0..t1 (contiguous in shared memory, so one
// descriptor with N = 64 (t1 - t0 + 1) <= 256 covers them) lands in the
// contiguous level accumulators s+t0 .. s+t1.  The two s = 1 MMAs cover every
// level (2..9) and start them at the first K step.
__device__ __forceinline__ void issue_levels(uint32_t tmem, uint32_t abase, uint32_t bbase, uint32_t ks,
                                             bool first) {
#pragma unroll
  for (int sl = 1; sl <= oz::S; ++sl) {
#pragma unroll
    for (int t0 = 1; t0 <= oz::S + 1 - sl; t0 += 4) {
      const int t1 = min(t0 + 3, oz::S + 1 - sl);
      const uint32_t idesc = instr_desc(128, OG_N * (t1 - t0 + 1));
      const uint64_t ad = smem_desc(abase + (sl - 1) * A_PART + ks * 2 * LBO);
      const uint64_t bd = smem_desc(bbase + (t0 - 1) * B_PART + ks * 2 * LBO);
      umma(tmem + (sl + t0 - 2) * OG_N, ad, bd, idesc, (first && sl == 1) ? 0u : 1u);
    }
  }
}

// sum_g L_g 2^-7g for 16 columns of this thread's TMEM lane (every level exact)
__device__ __forceinline__ void combine16(uint32_t taddr, float *hi, float *lo) {
  oz::combine16<9>(taddr, OG_N, hi, lo);
}

struct Barriers {
  uint64_t *full, *full_b, *empty, *tfull, *tempty, *spare;
  uint32_t *tmem_slot;
  volatile int *abort_flag;
};

// after the stages the epilogue scratch (OG_EPI), then the barrier block:
// full[S] (unused), full_b[S] (the stage's bulk copies landed), empty[S] (its
// MMAs finished reading it), tfull, tempty, spare, the TMEM address and the
// abort flag
__device__ __forceinline__ Barriers carve(uint8_t *smem) {
  Barriers b;
  uint64_t *bars = (uint64_t *)(smem + OG_STAGES * OG_STAGE + OG_EPI);
  b.full = bars;
  b.full_b = bars + OG_STAGES;
  b.empty = bars + 2 * OG_STAGES;
  b.tfull = bars + 3 * OG_STAGES;
  b.tempty = b.tfull + 1;
  b.spare = b.tempty + 1;  // drain_mmas before TMEM is freed
  b.tmem_slot = (uint32_t *)(b.spare + 1);
  b.abort_flag = (volatile int *)(b.tmem_slot + 1);
  return b;
}

// ---------------------------------------------------------------- Gram
struct GramArgs {
  const uint8_t *adig;  // A digit tiles [row_tiles][kstages][S][A_PART] (k_oz_slice_cols<128>)
  const uint8_t *bdig;  // B digit tiles [col_tiles][kstages][S][B_PART] (k_oz_slice_cols<64>)
  uint32_t kstages;     // K stages of KC rows per column tile (chunks * STAGES_PER_CHUNK)
  uint32_t row_tiles, col_tiles, splits, chunks;
  double *part;  // [items][OG_N][128] unscaled partial sums
  int *status;
};

// item it: K range (split) it / tiles, then the (row tile, column tile) pair,
// column tile fastest; split sp covers chunks [sp chunks / splits, (sp + 1)
// chunks / splits)
__device__ __forceinline__ void gram_item(const GramArgs &a, uint32_t it, uint32_t &rt, uint32_t &ct, uint32_t &c0,
                                          uint32_t &c1) {
  const uint32_t tiles = a.row_tiles * a.col_tiles;
  const uint32_t sp = it / tiles, tile = it % tiles;
  rt = tile / a.col_tiles;
  ct = tile % a.col_tiles;
  c0 = (uint32_t)(((uint64_t)sp * a.chunks) / a.splits);
  c1 = (uint32_t)(((uint64_t)(sp + 1) * a.chunks) / a.splits);
}

__global__ void __launch_bounds__(OG_THREADS, 1) k_oz_gram(const GramArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const Barriers br = carve(smem);
  const uint32_t tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const uint32_t n_items = a.row_tiles * a.col_tiles * a.splits;
  if (tid == 0) {
    for (int s = 0; s < OG_STAGES; ++s) {
      mbar_init(&br.full_b[s], 1);
      mbar_init(&br.empty[s], 1);
    }
    mbar_init(br.tfull, 1);
    mbar_init(br.tempty, PW);
    mbar_init(br.spare, 1);
    *br.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == PW + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(br.tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *br.tmem_slot;
  auto wait = [&](uint64_t *bar, uint32_t parity, int code) -> bool {
    if (*br.abort_flag) return false;
    if (mbar_wait(bar, parity, a.status, code)) return true;
    *br.abort_flag = 1;
    return false;
  };

  if (warp == PW) {
    // ---------------- bulk copies of the A and B digit tiles of each K stage
    if (lane == 0) {
      uint32_t q = 0;
      bool ok = true;
      for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        uint32_t rt, ct, c0, c1;
        gram_item(a, it, rt, ct, c0, c1);
        for (uint32_t kc = c0 * STAGES_PER_CHUNK; kc < c1 * STAGES_PER_CHUNK; ++kc, ++q) {
          const uint32_t s = q % OG_STAGES;
          if (q >= OG_STAGES && !wait(&br.empty[s], ((q / OG_STAGES) - 1) & 1, 40)) {
            ok = false;
            break;
          }
          uint8_t *At = smem + s * OG_STAGE;
          uint8_t *Bt = At + oz::S * A_PART;
          mbar_arrive_expect_tx(&br.full_b[s], oz::S * (A_PART + B_PART));
          const uint8_t *asrc = a.adig + ((uint64_t)rt * a.kstages + kc) * (oz::S * A_PART);
          const uint8_t *bsrc = a.bdig + ((uint64_t)ct * a.kstages + kc) * (oz::S * B_PART);
          for (int sl = 0; sl < oz::S; ++sl) {
            bulk_g2s(At + sl * A_PART, asrc + sl * A_PART, A_PART, &br.full_b[s]);
            bulk_g2s(Bt + sl * B_PART, bsrc + sl * B_PART, B_PART, &br.full_b[s]);
          }
        }
      }
      drain_copies(br.full_b, q, OG_STAGES);
    }
    __syncwarp();
  } else if (warp == PW + 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      uint32_t q = 0, nchunk = 0;
      bool ok = true;
      for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        uint32_t rt, ct, c0, c1;
        gram_item(a, it, rt, ct, c0, c1);
        for (uint32_t c = c0; c < c1 && ok; ++c, ++nchunk) {
          if (nchunk >= 1 && !wait(br.tempty, (nchunk - 1) & 1, 41)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          for (uint32_t st = 0; st < STAGES_PER_CHUNK; ++st, ++q) {
            const uint32_t s = q % OG_STAGES;
            if (!wait(&br.full_b[s], (q / OG_STAGES) & 1, 42)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t abase = smem_u32(smem + s * OG_STAGE);
            const uint32_t bbase = abase + oz::S * A_PART;
            for (uint32_t ks = 0; ks < KC / 16; ++ks) issue_levels(tmem, abase, bbase, ks, st == 0 && ks == 0);
            umma_commit(&br.empty[s]);
          }
          if (ok) umma_commit(br.tfull);
        }
      }
      drain_mmas(br.spare);
    }
    __syncwarp();
  } else if (warp < PW) {
    // ---------------- drains: after every 512-row chunk, TMEM -> FP64 registers
    const uint32_t quad = warp % 4, colh = warp / 4;
    uint32_t nchunk = 0;
    bool ok = true;
    for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
      uint32_t rt, ct, c0, c1;
      gram_item(a, it, rt, ct, c0, c1);
      double acc[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) acc[i] = 0.0;
      for (uint32_t c = c0; c < c1; ++c, ++nchunk) {
        ok = __all_sync(0xffffffffu, wait(br.tfull, nchunk & 1, 44));
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int cg = 0; cg < 2; ++cg) {
          float hi[16], lo[16];
          combine16(tmem + ((quad * 32) << 16) + colh * 32 + cg * 16, hi, lo);
#pragma unroll
          for (int i = 0; i < 16; ++i) acc[cg * 16 + i] += oz::df_to_double(hi[i], lo[i]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(br.tempty);
      }
      if (!ok) break;
      // partial of this item: [col][row], rows across lanes (coalesced)
      double *dst = a.part + (uint64_t)it * TILE;
      const uint32_t row = quad * 32 + lane;
#pragma unroll
      for (int i = 0; i < 32; ++i) dst[(uint64_t)(colh * 32 + i) * 128 + row] = acc[i];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == PW + 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

// S_o[i + ma j] = 2^(aexp + bexp + 2) * sum over splits, in a fixed order:
// a block takes 32 consecutive entries (coalesced partial reads) with
// FINAL_GROUPS warps, warp g summing splits g, g + FINAL_GROUPS, ... in
// ascending order; then the group sums are added in group order
constexpr int FINAL_GROUPS = 8;
__global__ void __launch_bounds__(32 * FINAL_GROUPS) k_oz_gram_final(const double *__restrict__ part, uint32_t na,
                                                                   uint32_t ma, uint32_t mb, uint32_t row_tiles,
                                                                   uint32_t col_tiles, uint32_t splits,
                                                                   const int *__restrict__ aexp,
                                                                   const int *__restrict__ bexp, double *S0,
                                                                   double *S1) {
  __shared__ double red[FINAL_GROUPS][32];
  const uint64_t total = (uint64_t)na * ma * mb;
  const uint32_t lane = threadIdx.x % 32, g = threadIdx.x / 32;
  for (uint64_t base = (uint64_t)blockIdx.x * 32; base < total; base += (uint64_t)gridDim.x * 32) {
    const uint64_t t = base + lane;
    const uint32_t R = (uint32_t)(t % (na * ma));
    const uint32_t j = (uint32_t)(t / (na * ma));
    double s = 0.0;
    if (t < total) {
      const uint32_t rt = R / 128, r = R % 128, ct = j / OG_N, cj = j % OG_N;
      // item of (split sp, tile) is sp * tiles + tile (k_oz_gram's order)
      const uint64_t tiles = (uint64_t)row_tiles * col_tiles;
      const double *p = part + (uint64_t)(rt * col_tiles + ct) * TILE + (uint64_t)cj * 128 + r;
#pragma unroll 4
      for (uint32_t sp = g; sp < splits; sp += FINAL_GROUPS) s += __ldg(p + (uint64_t)sp * tiles * TILE);
    }
    red[g][lane] = s;
    __syncthreads();
    if (g == 0 && t < total) {
      double v = red[0][lane];
#pragma unroll
      for (int k = 1; k < FINAL_GROUPS; ++k) v += red[k][lane];
      const uint32_t i = R % ma;
      (R < ma ? S0 : S1)[i + (uint64_t)ma * j] = v * oz::pow2(aexp[R] + bexp[j] + 2);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- rotation
struct RotArgs {
  const uint8_t *adig[3];        // row digit tiles of operand o: [row tile][K stage][S][A_PART] (k_oz_slice_rows)
  double *out[3];
  const __nv_bfloat16 *Tdig[3];  // factor of operand o: [col tile][K chunk][slice][OG_N x KC]
  const int *texp[3];            // its per-column exponents [mo]
  uint32_t kchunks[3];           // its K stages
  uint32_t nops, mo;             // mo output columns
  uint64_t N;
  const int *rexp;  // [nops][N] row exponents (over both halves of a K = 2m operand)
  uint32_t row_tiles, col_tiles;
  int *status;
};

__global__ void __launch_bounds__(OG_THREADS, 1) k_oz_rot(const RotArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const Barriers br = carve(smem);
  uint64_t *full_b = br.full_b;
  const uint32_t tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const uint32_t n_items = a.nops * a.row_tiles * a.col_tiles;
  if (tid == 0) {
    for (int s = 0; s < OG_STAGES; ++s) {
      mbar_init(&full_b[s], 1);
      mbar_init(&br.empty[s], 1);
    }
    mbar_init(br.tfull, 1);
    mbar_init(br.tempty, PW);
    mbar_init(br.spare, 1);
    *br.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == PW + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(br.tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *br.tmem_slot;
  auto wait = [&](uint64_t *bar, uint32_t parity, int code) -> bool {
    if (*br.abort_flag) return false;
    if (mbar_wait(bar, parity, a.status, code)) return true;
    *br.abort_flag = 1;
    return false;
  };
  // item it: (operand, row tile, column tile), column tile fastest, so the
  // CTAs reading the same row digit tiles run side by side (L2 reuse)
  auto decode = [&](uint32_t it, uint32_t &op, uint32_t &rt, uint32_t &ct) {
    ct = it % a.col_tiles;
    const uint32_t r = it / a.col_tiles;
    rt = r % a.row_tiles;
    op = r / a.row_tiles;
  };

  if (warp == PW) {
    // ---------------- bulk copies: row digit tiles and factor tiles
    if (lane == 0) {
      uint32_t q = 0;
      for (uint32_t it = blockIdx.x; it < n_items && !*br.abort_flag; it += gridDim.x) {
        uint32_t op, rt, ct;
        decode(it, op, rt, ct);
        const uint32_t nk = a.kchunks[op];
        bool ok = true;
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          const uint32_t s = q % OG_STAGES;
          if (q >= OG_STAGES && !wait(&br.empty[s], ((q / OG_STAGES) - 1) & 1, 51)) {
            ok = false;
            break;
          }
          uint8_t *At = smem + s * OG_STAGE;
          uint8_t *Bt = At + oz::S * A_PART;
          mbar_arrive_expect_tx(&full_b[s], oz::S * (A_PART + B_PART));
          const uint8_t *asrc = a.adig[op] + ((uint64_t)rt * nk + kc) * (oz::S * A_PART);
          const __nv_bfloat16 *bsrc = a.Tdig[op] + ((uint64_t)(ct * nk + kc) * oz::S) * (OG_N * KC);
          for (int sl = 0; sl < oz::S; ++sl) {
            bulk_g2s(At + sl * A_PART, asrc + sl * A_PART, A_PART, &full_b[s]);
            bulk_g2s(Bt + sl * B_PART, bsrc + (uint64_t)sl * OG_N * KC, B_PART, &full_b[s]);
          }
        }
        if (!ok) break;
      }
      drain_copies(full_b, q, OG_STAGES);
    }
    __syncwarp();
  } else if (warp == PW + 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      uint32_t q = 0, li = 0;
      bool ok = true;
      for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x, ++li) {
        if (li >= 1 && !wait(br.tempty, (li - 1) & 1, 52)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t nk = a.kchunks[it / (a.row_tiles * a.col_tiles)];
        for (uint32_t kc = 0; kc < nk; ++kc, ++q) {
          const uint32_t s = q % OG_STAGES;
          if (!wait(&full_b[s], (q / OG_STAGES) & 1, 54)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t abase = smem_u32(smem + s * OG_STAGE);
          const uint32_t bbase = abase + oz::S * A_PART;
          for (uint32_t ks = 0; ks < KC / 16; ++ks) issue_levels(tmem, abase, bbase, ks, kc == 0 && ks == 0);
          umma_commit(&br.empty[s]);
        }
        if (!ok) break;
        umma_commit(br.tfull);
      }
      drain_mmas(br.spare);
    }
    __syncwarp();
  } else {
    // ---------------- epilogue: levels -> FP64, scaled, whole-row-segment stores
    const uint32_t quad = warp % 4, colh = warp / 4;
    uint32_t li = 0;
    bool ok = true;
    for (uint32_t it = blockIdx.x; it < n_items && ok; it += gridDim.x, ++li) {
      uint32_t op, rt, ct;
      decode(it, op, rt, ct);
      ok = __all_sync(0xffffffffu, wait(br.tfull, li & 1, 56));
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t orow = (uint64_t)rt * 128 + quad * 32 + lane;
      const int oe = orow < a.N ? a.rexp[(uint64_t)op * a.N + orow] : 0;
      double *scr = (double *)(smem + OG_STAGES * OG_STAGE) + warp * oz::EPI_SCRATCH_DOUBLES;
#pragma unroll 1
      for (int cg = 0; cg < 2; ++cg) {
        const uint32_t j0 = ct * OG_N + colh * 32 + cg * 16;
        int te[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) te[i] = (j0 + i < a.mo) ? a.texp[op][j0 + i] : 0;
        oz::combine16_to_scratch(tmem + ((quad * 32) << 16) + colh * 32 + cg * 16, OG_N, scr, lane, oe, te);
        const uint32_t j = lane % 16;
#pragma unroll 4
        for (uint32_t i = 0; i < 16; ++i) {
          const uint32_t r = 2 * i + lane / 16;
          const uint64_t grow = (uint64_t)rt * 128 + quad * 32 + r;
          if (grow < a.N && j0 + j < a.mo) a.out[op][grow * a.mo + j0 + j] = oz::scratch_at(scr, r, j);
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(br.tempty);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == PW + 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

// ---------------------------------------------------------------- exponents and factor slices
// per-column exponents of up to two N x m blocks (stacked), two-stage max of
// the exponent bits (integer instructions: the FP64 pipe is the slow one)
__global__ void k_oz_colmax_partial(const double *__restrict__ A0, const double *__restrict__ A1, uint32_t na,
                                    uint32_t m, uint64_t N, int *__restrict__ part) {
  oz::colmax_partial_block(A0, A1, na, m, N, part);
}

__global__ void k_oz_colmax_final(const int *__restrict__ part, uint32_t nb, uint32_t cols, int *__restrict__ ex) {
  oz::colmax_final_block(part, nb, cols, ex);
}

// per-row exponents of the rotation inputs: one warp per row.  pair12: two
// operands, the second made of the rows of Y1 and Y2 side by side.
__global__ void k_oz_rowexp(const double *__restrict__ Y0, const double *__restrict__ Y1,
                            const double *__restrict__ Y2, uint32_t nops, uint32_t m, uint64_t N, bool pair12,
                            int *__restrict__ rexp) {
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
  const uint32_t lane = threadIdx.x % 32;
  for (uint64_t w = blockIdx.x * (uint64_t)(blockDim.x / 32) + threadIdx.x / 32; w < (uint64_t)nops * N; w += nw) {
    const uint32_t op = (uint32_t)(w / N);
    const uint64_t row = w - (uint64_t)op * N;
    const double *Y = op == 0 ? Y0 : (op == 1 ? Y1 : Y2);
    int mx = oz::EXP_NONE;
    for (uint32_t j = lane; j < m; j += 32) mx = max(mx, oz::exp_bits(Y[row * m + j]));
    if (pair12 && op == 1)
      for (uint32_t j = lane; j < m; j += 32) mx = max(mx, oz::exp_bits(Y2[row * m + j]));
    mx = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0) rexp[w] = oz::exp_or_zero(mx);
  }
}

// entry (i, j) of the factor: T (m x mo, column-major), or with neg_scale the
// 2m x mo factor [T; -T diag(neg_scale)]
__device__ __forceinline__ double factor_at(const double *__restrict__ T, const double *__restrict__ neg_scale,
                                            uint32_t m, uint32_t i, uint32_t j) {
  return i < m ? T[i + (uint64_t)m * j] : -(T[(i - m) + (uint64_t)m * j] * neg_scale[j]);
}

// slices of the factor as the B operand (rows = output columns j, K = input
// index i) with per-column exponents.  Block (column tile, K chunk): the four
// thread quarters take every fourth row of the column maxima (the whole K
// range, so every chunk's block finds the same exponents), then the block
// cuts its chunk; the first chunk's block stores the exponents.
__global__ void __launch_bounds__(256) k_oz_build_t(const double *__restrict__ T, const double *__restrict__ neg_scale,
                                                    uint32_t m, uint32_t mo, uint32_t kchunks, int *__restrict__ texp,
                                                    __nv_bfloat16 *__restrict__ out) {
  __shared__ double cmax[4][OG_N];
  __shared__ int cexp[OG_N];
  const uint32_t ct = blockIdx.x, kc = blockIdx.y;
  const uint32_t K = neg_scale ? 2 * m : m;
  {
    const uint32_t jr = threadIdx.x % OG_N, qt = threadIdx.x / OG_N;
    const uint32_t j = ct * OG_N + jr;
    double mx = 0.0;
    if (j < mo)
      for (uint32_t i = qt; i < K; i += 4) mx = fmax(mx, fabs(factor_at(T, neg_scale, m, i, j)));
    cmax[qt][jr] = mx;
  }
  __syncthreads();
  if (threadIdx.x < OG_N) {
    const uint32_t jr = threadIdx.x, j = ct * OG_N + jr;
    const double mx = fmax(fmax(cmax[0][jr], cmax[1][jr]), fmax(cmax[2][jr], cmax[3][jr]));
    cexp[jr] = oz::exponent_of(mx);
    if (kc == 0 && j < mo) texp[j] = cexp[jr];
  }
  __syncthreads();
  const uint32_t per_slice = OG_N * KC;
  __nv_bfloat16 *base = out + ((uint64_t)(ct * kchunks + kc) * oz::S) * per_slice;
  for (uint32_t rem = threadIdx.x; rem < per_slice; rem += blockDim.x) {
    const uint32_t jr = rem / KC, kk = rem % KC;
    const uint32_t j = ct * OG_N + jr, i = kc * KC + kk;
    int d[oz::S] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (j < mo && i < K) oz::digits(factor_at(T, neg_scale, m, i, j), cexp[jr], d);
    const uint32_t pos = (jr / 8) * (KC / 8) * 64 + (kk / 8) * 64 + (jr % 8) * 8 + (kk % 8);
#pragma unroll
    for (int s2 = 0; s2 < oz::S; ++s2) base[(uint64_t)s2 * per_slice + pos] = __int2bfloat16_rn(d[s2]);
  }
}

void set_attrs_once(int device) {
  static PerDeviceOnce once;
  once.run(device, [] {
    GBFE_CUDA(cudaFuncSetAttribute(k_oz_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OG_SMEM));
    GBFE_CUDA(cudaFuncSetAttribute(k_oz_rot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OG_SMEM));
  });
}

}  // namespace

namespace gbfe {

bool oz_gemm_supported(gbfe_ctx *ctx, uint32_t m) {
  return ctx->cc_major >= 10 && m > 0 && m <= (uint32_t)oz::K_EXACT;
}

// Item count of the Gram product: splits of the K range per (row tile, col
// tile) pair such that tiles x splits is a multiple of the SM count (every
// SM gets the same number of items), with at least one 512-row chunk per
// split where the K range allows it
static uint32_t gram_splits(uint32_t tiles, uint32_t chunks, uint32_t sms) {
  const uint32_t lo = std::max<uint32_t>(1, (sms + tiles - 1) / tiles);
  for (uint32_t sp = lo; sp <= std::min<uint32_t>(chunks, 8 * lo); ++sp)
    if (((uint64_t)tiles * sp) % sms == 0) return sp;
  return std::min(lo, std::max<uint32_t>(1, chunks));
}

// S_o (ma x mb, column-major) = A_o^T B for o < na (na <= 2); A_o: N x ma, B: N x mb, row-major blocks.
// bexp: the per-column exponents of B computed beforehand (nullptr: here)
void oz_gram(gbfe_ctx *ctx, const double *const *A, uint32_t na, uint32_t ma, const double *B, uint32_t mb,
             uint64_t N, double *const *S, const int *bexp) {
  GBFE_REQUIRE(na >= 1 && na <= 2 && ma > 0 && mb > 0, "oz_gram: bad shape");
  set_attrs_once(ctx->device);
  const uint32_t rows = na * ma;
  const uint32_t row_tiles = (rows + 127) / 128, col_tiles = (mb + OG_N - 1) / OG_N;
  const uint32_t chunks = (uint32_t)std::max<uint64_t>(1, (N + CHUNK - 1) / CHUNK);
  const uint32_t kstages = chunks * STAGES_PER_CHUNK;
  const uint32_t tiles = row_tiles * col_tiles;
  const uint32_t splits = gram_splits(tiles, chunks, (uint32_t)ctx->sm_count);
  const uint32_t items = tiles * splits;
  // exponents
  const unsigned nb = (unsigned)std::min<uint64_t>(8 * (uint64_t)ctx->sm_count, std::max<uint64_t>(1, N));
  ctx->oz_exp.ensure((size_t)rows + mb);
  ctx->oz_ipart.ensure((size_t)nb * std::max(rows, mb));
  k_oz_colmax_partial<<<nb, oz::COLMAX_THREADS, 0, ctx->stream>>>(A[0], na > 1 ? A[1] : A[0], na, ma, N,
                                                                  ctx->oz_ipart.p);
  k_oz_colmax_final<<<(rows + 31) / 32, oz::COLMAX_FINAL_THREADS, 0, ctx->stream>>>(ctx->oz_ipart.p, nb, rows,
                                                                                    ctx->oz_exp.p);
  count_launch(ctx, 2);
  if (bexp) {
    GBFE_CUDA(cudaMemcpyAsync(ctx->oz_exp.p + rows, bexp, sizeof(int) * mb, cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    k_oz_colmax_partial<<<nb, oz::COLMAX_THREADS, 0, ctx->stream>>>(B, B, 1, mb, N, ctx->oz_ipart.p);
    k_oz_colmax_final<<<(mb + 31) / 32, oz::COLMAX_FINAL_THREADS, 0, ctx->stream>>>(ctx->oz_ipart.p, nb, mb,
                                                                                    ctx->oz_exp.p + rows);
    count_launch(ctx, 2);
  }
  // the digit tiles of both operands, each value cut once
  const uint64_t a_bytes = (uint64_t)row_tiles * kstages * oz::S * A_PART;
  const uint64_t b_bytes = (uint64_t)col_tiles * kstages * oz::S * B_PART;
  ctx->oz_dig.ensure(a_bytes + b_bytes);
  uint8_t *adig = ctx->oz_dig.p, *bdig = ctx->oz_dig.p + a_bytes;
  {
    ProfScope prof(ctx, "slice_f64_oz", 0.0, 8.0 * (double)N * (rows + mb) + (double)(a_bytes + b_bytes));
    const uint64_t ta = (uint64_t)row_tiles * kstages, tb = (uint64_t)col_tiles * kstages;
    const unsigned gs = (unsigned)(ctx->sm_count * 8);
    k_oz_slice_cols<128><<<(unsigned)std::min<uint64_t>(ta, gs), 256, 0, ctx->stream>>>(
        A[0], na > 1 ? A[1] : A[0], ma, rows, N, ctx->oz_exp.p, kstages, ta, adig);
    k_oz_slice_cols<64><<<(unsigned)std::min<uint64_t>(tb, gs), 256, 0, ctx->stream>>>(
        B, B, mb, mb, N, ctx->oz_exp.p + rows, kstages, tb, bdig);
    check_launch(ctx, "oz_slice_cols");
    count_launch(ctx, 1);
  }
  ctx->oz_part.ensure((size_t)items * TILE);
  GramArgs args{adig, bdig, kstages, row_tiles, col_tiles, splits, chunks, ctx->oz_part.p, ctx->status.p};
  const uint32_t grid = std::min<uint32_t>(items, (uint32_t)ctx->sm_count);
  {
    ProfScope prof(ctx, "gram_f64_oz", 2.0 * (double)N * rows * mb, 8.0 * (double)N * (rows + mb));
    k_oz_gram<<<grid, OG_THREADS, OG_SMEM, ctx->stream>>>(args);
    check_launch(ctx, "oz_gram");
  }
  const uint64_t total = (uint64_t)rows * mb;
  k_oz_gram_final<<<(unsigned)std::min<uint64_t>((total + 31) / 32, (uint64_t)ctx->sm_count * 8), 32 * FINAL_GROUPS, 0,
                    ctx->stream>>>(ctx->oz_part.p, na, ma, mb, row_tiles, col_tiles, splits, ctx->oz_exp.p,
                                   ctx->oz_exp.p + rows, S[0], na > 1 ? S[1] : S[0]);
  check_launch(ctx, "oz_gram_final");
}

// Row exponents and row digit tiles of the rotation inputs (they depend on Y
// alone, so a caller can issue this before T is known).  Operand o < nops is
// Y[o] (K = m); with pair12 there are two operands, Y[0] (K = m) and the rows
// of Y[1], Y[2] side by side (K = 2m), as oz_rotate_residual takes them.
// Operand o's tiles start at byte rot_dig_offset(o) of ctx->oz_dig.
static uint64_t rot_tiles_bytes(uint64_t N, uint32_t K) {
  return ((N + 127) / 128) * (uint64_t)((K + KC - 1) / KC) * oz::S * A_PART;
}

void oz_rotate_rows(gbfe_ctx *ctx, const double *const *Y, uint32_t m, uint32_t nops, uint64_t N, bool pair12,
                    cudaStream_t stream) {
  if (pair12) nops = 2;
  const bool own = !stream || stream == ctx->stream;
  if (!stream) stream = ctx->stream;
  ctx->oz_rexp.ensure((size_t)nops * N);
  k_oz_rowexp<<<(unsigned)std::min<uint64_t>((nops * N + 7) / 8, (uint64_t)ctx->sm_count * 32), 256, 0, stream>>>(
      Y[0], nops > 1 ? Y[1] : Y[0], (nops > 2 || pair12) ? Y[2] : Y[0], nops, m, N, pair12, ctx->oz_rexp.p);
  count_launch(ctx, 1);
  uint64_t total = 0;
  for (uint32_t o = 0; o < nops; ++o) total += rot_tiles_bytes(N, (pair12 && o == 1) ? 2 * m : m);
  ctx->oz_dig.ensure(total);
  std::unique_ptr<ProfScope> prof;
  if (own)
    prof = std::make_unique<ProfScope>(ctx, "slice_f64_oz", 0.0,
                                       (double)N * m * 8.0 * (pair12 ? 3 : nops) + (double)total);
  uint64_t off = 0;
  for (uint32_t o = 0; o < nops; ++o) {
    const bool two = pair12 && o == 1;
    const uint32_t K = two ? 2 * m : m, kchunks = (K + KC - 1) / KC;
    const uint64_t ntiles = ((N + 127) / 128) * (uint64_t)kchunks;
    k_oz_slice_rows<<<(unsigned)std::min<uint64_t>(ntiles, (uint64_t)ctx->sm_count * 8), 256, 0, stream>>>(
        Y[o], two ? Y[2] : Y[o], m, K, N, ctx->oz_rexp.p + (uint64_t)o * N, kchunks, ntiles, ctx->oz_dig.p + off);
    off += rot_tiles_bytes(N, K);
  }
  check_launch(ctx, "oz_slice_rows");
  count_launch(ctx, nops - 1);
}

void oz_rotate(gbfe_ctx *ctx, const double *T, uint32_t m, uint32_t mo, const double *const *Y, double *const *out,
               uint32_t nops, uint64_t N, bool rows_ready) {
  GBFE_REQUIRE(nops >= 1 && nops <= 3 && m > 0 && m <= (uint32_t)oz::K_EXACT && mo > 0, "oz_rotate: bad shape");
  set_attrs_once(ctx->device);
  const uint32_t kchunks = (m + KC - 1) / KC, col_tiles = (mo + OG_N - 1) / OG_N;
  const uint32_t row_tiles = (uint32_t)((N + 127) / 128);
  ctx->oz_exp.ensure(mo);
  ctx->oz_tdig.ensure((size_t)col_tiles * kchunks * oz::S * OG_N * KC);
  if (!rows_ready) oz_rotate_rows(ctx, Y, m, nops, N, false);
  k_oz_build_t<<<dim3(col_tiles, kchunks), 256, 0, ctx->stream>>>(T, nullptr, m, mo, kchunks, ctx->oz_exp.p,
                                                                   ctx->oz_tdig.p);
  count_launch(ctx, 1);
  RotArgs args{};
  for (uint32_t o = 0; o < nops; ++o) {
    args.adig[o] = ctx->oz_dig.p + (uint64_t)o * rot_tiles_bytes(N, m);
    args.out[o] = out[o];
    args.Tdig[o] = ctx->oz_tdig.p;
    args.texp[o] = ctx->oz_exp.p;
    args.kchunks[o] = kchunks;
  }
  args.nops = nops;
  args.mo = mo;
  args.N = N;
  args.rexp = ctx->oz_rexp.p;
  args.row_tiles = row_tiles;
  args.col_tiles = col_tiles;
  args.status = ctx->status.p;
  const uint32_t items = nops * row_tiles * col_tiles;
  const uint32_t grid = std::min<uint32_t>(items, (uint32_t)ctx->sm_count);
  ProfScope prof(ctx, "rotate_f64_oz", 2.0 * (double)N * m * mo * nops, 8.0 * (double)N * (m + mo) * nops);
  k_oz_rot<<<grid, OG_THREADS, OG_SMEM, ctx->stream>>>(args);
  check_launch(ctx, "oz_rotate");
}

bool oz_rotate_residual_supported(gbfe_ctx *ctx, uint32_t m) { return oz_gemm_supported(ctx, 2 * m); }

// X = Y T and R = HY T - MY T diag(eps) (all N x m row-major, T m x m
// column-major, eps on the device) in one launch: R is the product of the rows
// [HY | MY] (K = 2m) with the factor [T; -T diag(eps)], so the rotated HY and
// MY are never stored.  rows_ready: oz_rotate_rows(..., pair12 = true) ran on
// these blocks already.
void oz_rotate_residual(gbfe_ctx *ctx, const double *T, const double *eps, uint32_t m, const double *Y,
                        const double *HY, const double *MY, double *X, double *R, uint64_t N, bool rows_ready) {
  GBFE_REQUIRE(m > 0 && oz_rotate_residual_supported(ctx, m), "oz_rotate_residual: bad shape");
  set_attrs_once(ctx->device);
  const uint32_t k0 = (m + KC - 1) / KC, k1 = (2 * m + KC - 1) / KC, col_tiles = (m + OG_N - 1) / OG_N;
  const uint32_t row_tiles = (uint32_t)((N + 127) / 128);
  const size_t fac0 = (size_t)col_tiles * k0 * oz::S * OG_N * KC;
  ctx->oz_exp.ensure(2 * (size_t)m);
  ctx->oz_tdig.ensure(fac0 + (size_t)col_tiles * k1 * oz::S * OG_N * KC);
  const double *in[3] = {Y, HY, MY};
  if (!rows_ready) oz_rotate_rows(ctx, in, m, 3, N, true);
  k_oz_build_t<<<dim3(col_tiles, k0), 256, 0, ctx->stream>>>(T, nullptr, m, m, k0, ctx->oz_exp.p, ctx->oz_tdig.p);
  k_oz_build_t<<<dim3(col_tiles, k1), 256, 0, ctx->stream>>>(T, eps, m, m, k1, ctx->oz_exp.p + m,
                                                             ctx->oz_tdig.p + fac0);
  count_launch(ctx, 2);
  RotArgs args{};
  args.adig[0] = ctx->oz_dig.p;
  args.adig[1] = ctx->oz_dig.p + rot_tiles_bytes(N, m);
  args.out[0] = X;
  args.out[1] = R;
  args.Tdig[0] = ctx->oz_tdig.p;
  args.Tdig[1] = ctx->oz_tdig.p + fac0;
  args.texp[0] = ctx->oz_exp.p;
  args.texp[1] = ctx->oz_exp.p + m;
  args.kchunks[0] = k0;
  args.kchunks[1] = k1;
  args.nops = 2;
  args.mo = m;
  args.N = N;
  args.rexp = ctx->oz_rexp.p;
  args.row_tiles = row_tiles;
  args.col_tiles = col_tiles;
  args.status = ctx->status.p;
  const uint32_t items = 2 * row_tiles * col_tiles;
  const uint32_t grid = std::min<uint32_t>(items, (uint32_t)ctx->sm_count);
  ProfScope prof(ctx, "rotate_f64_oz", 6.0 * (double)N * m * m, 40.0 * (double)N * m);
  k_oz_rot<<<grid, OG_THREADS, OG_SMEM, ctx->stream>>>(args);
  check_launch(ctx, "oz_rotate_residual");
}

}  // namespace gbfe
