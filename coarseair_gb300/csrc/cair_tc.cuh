// Fifth-generation tensor-core primitives for sm_103a, written as inline PTX: tensor-memory (TMEM)
// allocation, tcgen05.mma of BF16 operands with FP32 accumulation in TMEM, completion through an
// mbarrier, and TMEM loads of a CTA's accumulator rows.
//
// Operands are staged in shared memory by the CTA's own threads (st.shared) in the canonical
// no-swizzle layouts: an 8-row x 16-byte core matrix is 128 contiguous bytes, and the descriptor's
// two byte offsets step between core matrices along K and along M/N.  With M = 128 and
// cta_group::1 the accumulator row r is TMEM lane r, so thread r of a 128-thread CTA reads its own
// row: the per-row epilogue (bias, activation, the next layer's operand) stays in that thread.
//
// Every wait is bounded: an mbarrier wait gives up after kWaitNs of %globaltimer (and an
// iteration cap), reports it through the caller's error flag and returns; the caller then skips
// the work that depended on it, drains, frees its TMEM and exits.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace cair {
namespace tc {

constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s
constexpr unsigned kWaitIters = 1u << 28;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- TMEM allocation (one whole warp) ----
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- ordering ----
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of the given parity; false if it did not complete within the bound.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (unsigned it = 0; it < kWaitIters; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && globaltimer() - t0 > kWaitNs) return false;
  }
  return false;
}

// ---- MMA ----
// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, dense: D format bits 4-5 (1 = F32),
// A format 7-9 and B format 10-12 (1 = BF16), A major bit 15 and B major bit 16 (0 = K-major,
// 1 = MN-major), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool b_mn_major = false) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((b_mn_major ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Shared-memory matrix descriptor, no swizzle: start address >> 4 (bits 0-13), leading-dimension
// byte offset >> 4 (16-29), stride-dimension byte offset >> 4 (32-45), the fixed 0b001 of this
// descriptor version at bits 46-48, base offset 0, swizzle mode 0.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// D[tmem] (+)= A[smem] x B[smem]^T, one instruction (K = 16 for BF16); issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The mbarrier receives one arrival when every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---- TMEM -> registers: 16 consecutive 32-bit columns of the thread's lane ----
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- canonical no-swizzle layouts ----
// K-major operand X[rows][K] (rows = M or N): core matrix (r / 8, k / 8) at
// (k / 8) * rows * 16 + (r / 8) * 128, row r % 8 at 16-byte steps, element k % 8 at 2-byte steps.
// Descriptor: leading-dimension (K) offset rows * 16, stride-dimension (M/N) offset 128; the MMA of
// K-step s starts 2 * s * rows * 16 bytes in.
__host__ __device__ __forceinline__ uint32_t kmaj_off(int r, int k, int rows) {
  return (uint32_t)((k >> 3) * rows * 16 + (r >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// ---- exact three-way BF16 split of an FP32 value ----
// a = hi + mid + lo with each part a BF16 (round to nearest even at every step).  For |a| in the
// normal range the three parts hold a's 24 significant bits, so a BF16 x BF16 product of each part
// is exact in the FP32 accumulator and the sum of the three products is a x w to FP32 accumulation.
__device__ __forceinline__ void split3(float a, __nv_bfloat16& hi, __nv_bfloat16& mid, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(a);
  const float r1 = a - __bfloat162float(hi);
  mid = __float2bfloat16_rn(r1);
  lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
}

}  // namespace tc
}  // namespace cair
