// gbfe_tc_ptx.cuh -- tcgen05 / TMA / mbarrier building blocks shared by the
// tensor-core cell products (split-BF16 in gbfe_tc.cu, FP64-accurate sliced
// products in gbfe_ozaki.cu).  Operands use the canonical no-swizzle K-major
// layout: core matrices of 8 rows x 16 bytes, K-adjacent core matrices LBO
// bytes apart, 8-row groups SBO bytes apart.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace gbfe {
namespace tc {

constexpr int KC = 32;       // K extent of one pipeline stage (2 MMA K-steps)
constexpr int STAGES = 3;
constexpr int THREADS = 128;  // 4 warps: gather, epilogue; thread 0 issues TMA + MMA
constexpr uint32_t CORE_BYTES = 128;             // one 8 x 16-byte core matrix
constexpr uint32_t SBO = (KC / 8) * CORE_BYTES;  // stride between 8-row groups
constexpr uint32_t LBO = CORE_BYTES;             // stride between K-adjacent core matrices
constexpr uint32_t WAIT_LIMIT = 1u << 24;        // bounded mbarrier polls
constexpr uint64_t WAIT_NS = 2000000000ull;      // and at most 2 s per wait
constexpr uint32_t WAIT_SUSPEND_NS = 20000;      // a poll may suspend the thread this long (woken at completion)

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

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait on the given phase parity (max_polls polls and max_ns of wall
// time, whichever ends first); false on timeout, and then, when status is
// given, the error code goes into the device status word
__device__ __forceinline__ bool mbar_wait_limited(uint64_t *bar, uint32_t parity, int *status, int code,
                                                  uint32_t max_polls, uint64_t max_ns) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0;
  for (uint32_t it = 0; it < max_polls; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(WAIT_SUSPEND_NS)
        : "memory");
    if (ok) return true;
    if ((it & 255u) == 255u) {
      const uint64_t t = globaltimer_ns();
      if (!t0)
        t0 = t;
      else if (t - t0 > max_ns)
        break;
    }
  }
  if (status) atomicCAS(status, 0, code);
  return false;
}

// the waits of the tensor-core kernels: WAIT_LIMIT polls or WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *status, int code) {
  return mbar_wait_limited(bar, parity, status, code, WAIT_LIMIT, WAIT_NS);
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// L2 policy for data read once per launch (streamed operand tiles): evicted
// first, so the block vectors and cell-wise results other kernels read next
// stay in L2
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ void bulk_g2s_stream(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                                uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
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

// After a timed-out wait the CTA leaves its loops early; before it frees TMEM
// and exits, the asynchronous work its threads issued must have landed.
//   drain_copies: the bulk copies of the last min(q, S) ring chunks issued
//     (chunk j signals full[j % S], phase parity (j / S) & 1);
//   drain_mmas: every tcgen05.mma this thread issued (a commit to a spare
//     barrier that nothing else arrives on, used once).
// Both waits are bounded and leave the status word alone.
__device__ __forceinline__ void drain_copies(uint64_t *full, uint32_t q, uint32_t S) {
  for (uint32_t j = q > S ? q - S : 0; j < q; ++j) mbar_wait(&full[j % S], (j / S) & 1, nullptr, 0);
}
__device__ __forceinline__ void drain_mmas(uint64_t *spare) {
  umma_commit(spare);
  mbar_wait(spare, 0, nullptr, 0);
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

// tcgen05.ld of 16 columns without the wait: tmem_wait_ld16 completes it.
// The destination registers are in/out operands of the wait, so no read of
// them is placed above it.
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld16(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 16-byte asynchronous global -> shared copy (L2 only); src_bytes 0 writes 16
// zero bytes and reads nothing.  Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void *dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most n of this thread's copy groups are pending (n < 4); the
// completed copies are then visible to this thread
__device__ __forceinline__ void cp_async_wait(uint32_t n) {
  if (n == 0)
    asm volatile("cp.async.wait_group 0;" ::: "memory");
  else if (n == 1)
    asm volatile("cp.async.wait_group 1;" ::: "memory");
  else if (n == 2)
    asm volatile("cp.async.wait_group 2;" ::: "memory");
  else
    asm volatile("cp.async.wait_group 3;" ::: "memory");
}

}  // namespace tc
}  // namespace gbfe
