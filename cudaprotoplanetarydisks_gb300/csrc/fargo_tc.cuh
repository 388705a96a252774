// fargo_tc.cuh -- 5th-generation tensor-core (tcgen05) building blocks for sm_103a:
// tensor-memory allocation, shared-memory matrix descriptors, the BF16 MMA with FP32
// accumulators in tensor memory, its completion on an mbarrier, and the loads of
// the accumulators back to registers.  Inline PTX only.
//
// Operand layout (no swizzle, K-major): a matrix of R rows x K columns (BF16) is
// stored as "core matrices" of 8 rows x 16 bytes (8 elements), each 128 contiguous
// bytes with its rows 16 bytes apart.  Element (r, k) sits at
//     (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// bytes from the matrix start: LBO is the distance between core matrices adjacent
// along K (the leading dimension), SBO between core matrices adjacent along the
// rows (the strided dimension).  The MMA reads A (M x K) and B (N x K) from such
// layouts and accumulates D (M x N, FP32) in tensor memory: lane m, column n.
//
// Every wait is bounded; a kernel that gives up reports it and still frees its
// tensor memory before it returns.
#pragma once
#include <cstdint>

namespace tc {

// shared-memory matrix descriptor (64 bits): start address >> 4 (bits 0-13), LBO >> 4
// (16-29), SBO >> 4 (32-45), descriptor version 1 (46-47), base offset 0 (49-51),
// absolute LBO mode off (52), layout 0 = no swizzle (61-63)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16 (32 bits): dense, no saturation, D = FP32
// (bits 4-5 = 1), A = BF16 (7-9 = 1), B = BF16 (10-12 = 1), no negation, A and B
// K-major (15, 16 = 0), N >> 3 (17-22), M >> 4 (24-28)
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tensor-memory allocation of ncols columns (a power of two, >= 32) by one whole
// warp; the address lands in shared memory at *slot
__device__ __forceinline__ void alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[taddr] (+)= A * B^T, issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
      ::"r"(taddr), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}
// the mbarrier at bar arrives once every MMA this thread issued so far has completed
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase `parity`: false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = 1u << 22) {
  for (uint32_t n = 0; n < limit; n++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 16 consecutive FP32 columns of this thread's lane (lane = the warp's quarter of
// the 128 lanes + lane id) starting at taddr; complete after wait_ld()
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of element (r, k) in the no-swizzle K-major layout
__host__ __device__ constexpr uint32_t kmajor_offset(int r, int k, uint32_t lbo, uint32_t sbo) {
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 3) * lbo + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

}  // namespace tc
