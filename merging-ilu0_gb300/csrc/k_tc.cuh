// Blackwell (sm_100a / sm_103a) tensor-core building blocks in inline PTX:
// tensor-memory (TMEM) allocation, tcgen05.mma with BF16 operands in shared
// memory and FP32 accumulators in TMEM, completion through an mbarrier, and
// tcgen05.ld of the accumulators back into registers.  Used by the learned
// warm start's 64x64 layers (k_mlp.cu); one CTA, no clusters, no TMA.
//
// Operand layout (no swizzle, K-major).  A matrix of R rows and K columns
// (BF16) is stored as 8-row x 16-byte core matrices: element (r, k) at byte
//     (r % 8) * 16 + (r / 8) * SBO + (k / 8) * 128 + (k % 8) * 2,   SBO = K * 16,
// so the 8 rows of one core matrix are 128 contiguous bytes, core matrices
// adjacent in K are 128 bytes apart (the descriptor's leading byte offset) and
// 8-row groups SBO bytes apart (its stride byte offset).  One MMA takes K = 16:
// the descriptor of k-step j starts 2 * 128 * j bytes into the matrix.
//
// Accumulator layout (M = 128, cta_group::1): row i of D in TMEM lane i,
// column j in TMEM column j (32-bit); warp w of the CTA reads lanes
// 32 (w % 4) .. 32 (w % 4) + 31, one row per thread.
#pragma once

#include <cstdint>

namespace bilu {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) of a K-major operand with K columns (see above).
__host__ __device__ constexpr uint32_t kmajor_off(int r, int k, int K) {
  return (uint32_t)((r & 7) * 16 + (r >> 3) * (K * 16) + (k >> 3) * 128 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading byte offset 128,
// stride byte offset sbo (all >> 4), descriptor version 1 (bits 46-47),
// base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((128u >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4
// at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM allocation of ncols columns (a power of two >= 32) by one whole warp;
// the address lands in *slot (shared memory).
__device__ __forceinline__ void alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) = A * B^T (+ D when accumulate), issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The mbarrier receives one arrival when every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Waits (non-blocking polls, at most `limit`) for the phase of parity `parity`
// to complete; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Orderings around thread barriers, and of generic-proxy shared-memory writes
// before the tensor core (async proxy) reads them.
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive 32-bit columns of this thread's TMEM lane (32x32b shape),
// waited for in the same statement, so no use of the registers can be
// scheduled before the load has completed.
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

}  // namespace tc
}  // namespace bilu
