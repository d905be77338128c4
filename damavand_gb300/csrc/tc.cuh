// Fifth-generation tensor-core (tcgen05) primitives, inline PTX for sm_103a.
//
// Used by the tensor-core window pass (DMV_ARITH_TC): one thread issues
// tcgen05.mma with both operands in shared memory, the accumulators live in
// tensor memory (TMEM, 128 lanes x 512 columns of 32 bits per SM) and the
// CTA's threads read them back with tcgen05.ld. Operands use the canonical
// K-major layout without swizzle: a "core matrix" is 8 rows x 16 bytes stored
// as 128 contiguous bytes; core matrices adjacent along K are LBO bytes apart
// and those adjacent along M/N are SBO bytes apart.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace dmv {

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1 (bit 46), no swizzle.
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16 with FP16 A and B (both K-major) and an
// FP32 accumulator: D format at bits 4-5, N/8 at bits 17-22, M/16 at 24-28.
__host__ __device__ constexpr uint32_t tc_idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// One warp allocates `ncols` TMEM columns (a power of two >= 32) and writes
// the base address to shared memory; the permit is released so other CTAs
// on the SM may allocate.
__device__ __forceinline__ void tc_alloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem_dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T; accumulate = 0 overwrites D.
__device__ __forceinline__ void tc_mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                           uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// True in exactly one lane of the (fully active) warp: the lowest.
__device__ __forceinline__ bool tc_elect_one() {
  uint32_t e;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "elect.sync _|p, 0xffffffff;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(e));
  return e != 0;
}

// Arrives (once) on `bar` when every tcgen05 operation this thread issued
// before has completed.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(bar))
               : "memory");
}

// Orders tcgen05 operations after (before) the thread synchronisation that
// follows (precedes) them.
__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// Thread i of the warp reads TMEM lane (lane base + i), 8 consecutive
// columns from `taddr`. Completes at tc_wait_ld.
__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace dmv
