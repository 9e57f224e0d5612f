// gbfe_oz.cuh -- shared pieces of the FP64-accurate sliced tensor-core
// products (the splitting scheme of Ozaki, Ogita, Oishi & Rump, Numer.
// Algorithms 59, 2012):
//
//   v = 2^(e+1) * sum_{s=1..8} d_s 2^(-7 s),   |v| < 2^e,  d_s integers in [-64, 64]
//
// The value is scaled to a 55-bit signed fixed-point integer (truncated:
// error below 2^(e-55)) and cut into balanced base-128 digits.  Every digit
// product is at most 2^12 in magnitude, so a level sum
// L_g = sum_{s+t=g} sum_k a_s x_t (at most 8 digit pairs) over K <= 512 terms
// stays within 2^24 and FP32 tensor-core accumulation of it is exact.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "gbfe_tc_ptx.cuh"

namespace gbfe {
namespace oz {

constexpr int S = 8;       // slices per operand
constexpr int LEVELS = 8;  // g = s + t = 2..9 (36 digit pairs); g >= 10 is below 2^-63 and dropped
constexpr int K_EXACT = 512;  // longest exact FP32 accumulation of one level

// smallest e with |v| < 2^e (0 for v == 0)
__device__ __forceinline__ int exponent_of(double vmax) {
  if (!(vmax > 0.0)) return 0;
  int e;
  frexp(vmax, &e);
  return e;
}

// exponent_of(|v|) from the bits alone (integer pipe): for a normal double of
// biased exponent E, |v| = 1.f 2^(E-1023) < 2^(E-1022).  Zero / subnormal
// give EXP_NONE, so max() over a set equals exponent_of(max |v|) whenever the
// set has a normal entry; finish with exp_or_zero().
constexpr int EXP_NONE = -100000;
__device__ __forceinline__ int exp_bits(double v) {
  const int E = (int)(((uint64_t)__double_as_longlong(v) >> 52) & 0x7ff);
  return E == 0 ? EXP_NONE : E - 1022;
}
__device__ __forceinline__ int exp_or_zero(int e) { return e == EXP_NONE ? 0 : e; }

// trunc(v 2^(55-e)) as a signed integer, |.| < 2^55 for |v| < 2^e
__device__ __forceinline__ int64_t fixed55(double v, int e) {
  const uint64_t bits = (uint64_t)__double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7ff);
  if (ex == 0) return 0;
  const uint64_t mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
  const int sh = ex - 1075 + 55 - e;  // v 2^(55-e) = mant 2^sh and |v| < 2^e: sh <= 2
  uint64_t fx = 0;
  if (sh >= 0)
    fx = mant << sh;
  else if (sh > -64)
    fx = mant >> (-sh);
  return (bits >> 63) ? -(int64_t)fx : (int64_t)fx;
}

// Balanced base-128 digits of v (|v| < 2^e), d[0] most significant.  Adding 64
// at each of the seven low digit positions turns the balanced digits b_j in
// [-64, 63] into the plain base-128 digits b_j + 64 of the sum, so every digit
// is one shift-and-mask; the top digit is the arithmetic shift of the rest
// (|d[0]| <= 64).
constexpr int64_t DIGIT_BIAS = 64LL * (((1LL << 49) - 1) / 127);
__device__ __forceinline__ void digits(double v, int e, int *d) {
  const int64_t Y = fixed55(v, e) + DIGIT_BIAS;
  const uint64_t u = (uint64_t)Y;
#pragma unroll
  for (int s = 1; s < S; ++s) d[s] = (int)((u >> (7 * (S - 1 - s))) & 127u) - 64;
  d[0] = (int)(Y >> 49);
}

// small integer -> float without the conversion unit (exact for |d| < 2^22)
__device__ __forceinline__ float int_to_float_small(int d) {
  return __int_as_float(0x4B400000 + d) - 12582912.0f;
}

// the 8 slices of two consecutive K values, packed as BF16 pairs (low half =
// first value): packed[s] for slice s.  A digit (|d| <= 64) is a float with
// at most 7 significant bits, so its BF16 form is the upper half of the float
// bits: one byte permute per pair, no conversion instruction.
__device__ __forceinline__ void digits_pair_bf16(double v0, double v1, int e, uint32_t *packed) {
  int d0[S], d1[S];
  digits(v0, e, d0);
  digits(v1, e, d1);
#pragma unroll
  for (int s = 0; s < S; ++s)
    packed[s] = __byte_perm(__float_as_uint(int_to_float_small(d0[s])), __float_as_uint(int_to_float_small(d1[s])),
                            0x7632);
}

// Stage 1 of the per-column exponent scan of up to two stacked N x m row-major
// blocks (column c < m of A0, else column c - m of A1): the block of this CTA's
// rows, max of the exponent bits per column into part[blockIdx.x][na m].
// Threads are (row lane, column) with consecutive threads on consecutive
// columns, so every pass reads whole rows; four rows per lane are loaded
// before they are reduced.  max is order-free: any split gives the same bits.
constexpr int COLMAX_THREADS = 256;
__device__ __forceinline__ void colmax_partial_block(const double *__restrict__ A0, const double *__restrict__ A1,
                                                     uint32_t na, uint32_t m, uint64_t N, int *__restrict__ part) {
  __shared__ int red[COLMAX_THREADS];
  const uint32_t cols = na * m;
  const uint64_t per = (N + gridDim.x - 1) / gridDim.x;
  const uint64_t r0 = blockIdx.x * per, r1 = min(N, r0 + per);
  const uint32_t tcols = min(cols, (uint32_t)COLMAX_THREADS), rpb = COLMAX_THREADS / tcols;
  const uint32_t rl = threadIdx.x / tcols, cl = threadIdx.x % tcols;
  for (uint32_t cb = 0; cb < cols; cb += tcols) {
    const uint32_t c = cb + cl;
    int mx = EXP_NONE;
    if (rl < rpb && c < cols) {
      const double *A = c < m ? A0 : A1;
      const uint32_t j = c < m ? c : c - m;
      uint64_t i = r0 + rl;
      for (; i + 3 * (uint64_t)rpb < r1; i += 4 * (uint64_t)rpb) {
        const double x0 = A[i * m + j], x1 = A[(i + rpb) * m + j], x2 = A[(i + 2 * rpb) * m + j],
                     x3 = A[(i + 3 * rpb) * m + j];
        mx = max(max(mx, max(exp_bits(x0), exp_bits(x1))), max(exp_bits(x2), exp_bits(x3)));
      }
      for (; i < r1; i += rpb) mx = max(mx, exp_bits(A[i * m + j]));
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    if (rl == 0 && c < cols) {
      for (uint32_t q = 1; q < rpb; ++q) mx = max(mx, red[q * tcols + cl]);
      part[(uint64_t)blockIdx.x * cols + c] = mx;
    }
    __syncthreads();
  }
}

// Stage 2: ex[c] = max over the nb partial rows, for 32 columns per CTA of
// COLMAX_FINAL_THREADS threads (32 row lanes x 32 columns, coalesced reads),
// the lanes' maxima combined through shared memory; EXP_NONE becomes 0.
constexpr int COLMAX_FINAL_THREADS = 1024;
__device__ __forceinline__ void colmax_final_block(const int *__restrict__ part, uint32_t nb, uint32_t cols,
                                                   int *__restrict__ ex) {
  __shared__ int red[COLMAX_FINAL_THREADS];
  const uint32_t cl = threadIdx.x % 32, rl = threadIdx.x / 32, rows = COLMAX_FINAL_THREADS / 32;
  const uint32_t c = blockIdx.x * 32 + cl;
  int mx = EXP_NONE;
  if (c < cols)
    for (uint32_t b = rl; b < nb; b += rows) mx = max(mx, part[(uint64_t)b * cols + c]);
  red[threadIdx.x] = mx;
  __syncthreads();
  if (rl == 0 && c < cols) {
    for (uint32_t q = 1; q < rows; ++q) mx = max(mx, red[q * 32 + cl]);
    ex[c] = exp_or_zero(mx);
  }
}

// out-of-line, so that the rare call is a branch and not FP64 work that the
// compiler predicates into every lane
static __device__ __noinline__ double ldexp_outlined(double v, int k) { return ldexp(v, k); }

// v * 2^k by adding k to the exponent field (integer pipe), exact; zero
// stays zero and results outside the normal range go through ldexp.
__device__ __forceinline__ double scale2(double v, int k) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return v;                                            // zero
  if (e + k <= 0 || e + k >= 0x7ff) return ldexp_outlined(v, k);  // leaves the normal range
  return __longlong_as_double(b + ((long long)k << 52));
}

// float -> double by moving the bit fields (integer pipe; the FP64 pipe is the
// scarce one).  Exact for zero and normal floats, which is all the level
// sums and their TwoSum errors can be (integer multiples of 2^-63 or zero).
__device__ __forceinline__ double f2d(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sign);
  return __longlong_as_double((long long)(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29)));
}

// hi + lo of a double-float as one FP64 add
__device__ __forceinline__ double df_to_double(float hi, float lo) { return f2d(hi) + f2d(lo); }

// 2^k as a double (k within the normal range)
__device__ __forceinline__ double pow2(int k) { return __longlong_as_double((long long)(uint64_t)(k + 1023) << 52); }

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// sum_g L_g 2^-7g of one accumulator column, smallest level first, as an
// FP32 double-float (every term L_g 2^-7g is exact in FP32)
__device__ __forceinline__ float level_weight(int g) { return __int_as_float((127 - 7 * g) << 23); }

// sum_g L_g 2^-7g (g = 9 .. 2, smallest level first) for 16 columns of this
// thread's TMEM lane; level g's accumulator at taddr + (g - 2) * stride.  The
// load of the next level is in flight while the current one is added.
// Levels 9, 8, 7 are summed with plain FP32 fused multiply-adds: with
// |L_g| <= K 2^15 their partial sum is below K 2^-34 and its two roundings
// below K 2^-57, i.e. 2^-55 of the product bound K/4 (in the same units); the
// operand truncation already contributes 2^-54.  Levels 6 .. 2 go through
// error-free TwoSums into the (hi, lo) pair.  EXACT_FROM = 9: every level
// through TwoSums (the Gram kernel: its FP64 chunk accumulators leave no
// registers for the shorter schedule).
template <int EXACT_FROM = 6>
__device__ __forceinline__ void combine16(uint32_t taddr, uint32_t stride, float *hi, float *lo) {
#pragma unroll
  for (int q = 0; q < 16; ++q) hi[q] = lo[q] = 0.f;
  uint32_t La[16], Lb[16];
  auto step = [&](uint32_t(&cur)[16], uint32_t(&nxt)[16], int g) {
    if (g > 2) tc::tmem_ld16_issue(taddr + (uint32_t)(g - 3) * stride, nxt);
    const float w = level_weight(g);
    if (g > EXACT_FROM) {
#pragma unroll
      for (int q = 0; q < 16; ++q) hi[q] = fmaf(__uint_as_float(cur[q]), w, hi[q]);
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float s2, e2;
        two_sum(hi[q], __uint_as_float(cur[q]) * w, s2, e2);
        hi[q] = s2;
        lo[q] += e2;
      }
    }
    if (g > 2) tc::tmem_wait_ld16(nxt);
  };
  tc::tmem_ld16_issue(taddr + (uint32_t)(S - 1) * stride, La);
  tc::tmem_wait_ld16(La);
  step(La, Lb, 9);
  step(Lb, La, 8);
  step(La, Lb, 7);
  step(Lb, La, 6);
  step(La, Lb, 5);
  step(Lb, La, 4);
  step(La, Lb, 3);
  step(Lb, La, 2);
}
static_assert(S + 1 == 9, "combine16 is written out for levels 9 .. 2");

// Epilogue staging of one warp (its 32 TMEM lanes = 32 output rows): 16
// columns are combined, scaled by 2^(row_e + col_e[j] + 2) and written into the
// warp's 32 x 16 FP64 scratch, entry (r, j) at r * 16 + (j ^ (r % 16)); the
// row-wise reads that follow (scratch_at) hand each half-warp 16 consecutive
// columns of one row, so the global stores are whole 128-byte row segments.
// Both the per-lane writes and the per-row reads touch every bank pair twice
// per warp access: no conflicts beyond the two wavefronts of 256 bytes.
constexpr uint32_t EPI_SCRATCH_DOUBLES = 32 * 16;  // per warp
__device__ __forceinline__ void combine16_to_scratch(uint32_t taddr, uint32_t stride, double *scratch, uint32_t lane,
                                                     int row_e, const int (&col_e)[16]) {
  float hi[16], lo[16];
  combine16(taddr, stride, hi, lo);
#pragma unroll
  for (int j = 0; j < 16; ++j)
    scratch[lane * 16 + (j ^ (lane & 15))] = scale2(df_to_double(hi[j], lo[j]), row_e + col_e[j] + 2);
  __syncwarp();
}
__device__ __forceinline__ double scratch_at(const double *scratch, uint32_t r, uint32_t j) {
  return scratch[r * 16 + (j ^ (r & 15))];
}

}  // namespace oz
}  // namespace gbfe
