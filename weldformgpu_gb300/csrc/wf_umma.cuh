// wf_umma.cuh — the Blackwell tensor-core (tcgen05, "UMMA") primitives the
// library uses, as inline PTX for sm_100a / sm_103a: tensor-memory
// allocation, the shared-memory matrix descriptor, the instruction descriptor
// of kind::f16 with BF16 operands and FP32 accumulation, the MMA, its commit
// to an mbarrier, bounded mbarrier waits, and 32x32b tensor-memory loads.
//
// Layout used for both operands: K-major without swizzle.  A "core matrix"
// is 8 rows x 16 bytes (8 BF16 values of K), stored contiguously (128 bytes).
// Element (row r, column k) of an operand with K columns sits at
//   (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2   bytes,
// with LBO = 128 (core matrices adjacent along K) and SBO = K * 16 (the next
// group of 8 rows).  One MMA consumes K = 16, i.e. two core matrices along K;
// the k-th step of a wider operand starts 256 bytes further on.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace umma {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, all >> 4; bit 46 is the fixed 0b001 field;
// base offset 0, relative LBO, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D = FP32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Tensor memory: one warp allocates ncols columns (a power of two >= 32)
// and writes the base address to shared memory; the same warp frees them.
// A CTA of a kernel that contains tcgen05.alloc holds an allocation permit
// until it relinquishes it, and while it holds it no further CTA of the
// kernel starts on its SM: every CTA relinquishes at entry, after its
// allocation or without one.
__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               :: "r"(slot_saddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void relinquish_permit() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
// the MMAs issued so far by this thread arrive on the mbarrier when done
__device__ __forceinline__ void commit(uint32_t mbar_saddr) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(mbar_saddr) : "memory");
}

// initialised by one thread; the fence makes the initialisation visible to
// the tensor core's arrive before the block barrier that follows
__device__ __forceinline__ void mbar_init(uint32_t mbar_saddr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(mbar_saddr), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Waits for phase `parity` to complete, at most `limit` polls; false when
// the limit ran out (the caller reports it and does not use the result).
__device__ __forceinline__ bool mbar_wait(uint32_t mbar_saddr, uint32_t parity, int limit) {
  for (int it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(mbar_saddr), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// One bulk copy (TMA, untiled) of `bytes` from global to shared memory whose
// completion is counted on the mbarrier: the issuing thread arrives once and
// announces the byte count.  Both addresses 16-byte aligned, bytes a
// multiple of 16.
__device__ __forceinline__ void bulk_load(uint32_t dst_saddr, const void* src, uint32_t bytes,
                                          uint32_t mbar_saddr) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               :: "r"(mbar_saddr), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      :: "r"(dst_saddr), "l"(src), "r"(bytes), "r"(mbar_saddr) : "memory");
}

// 16 consecutive 32-bit columns of the calling thread's tensor-memory lane
// (the warp's quadrant of lanes is fixed by the lane field of taddr).  The
// load and its wait are one asm statement, so no use of the registers can be
// scheduled before the data has arrived.
__device__ __forceinline__ void ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

}  // namespace umma
