// Blackwell (sm_100 / sm_103) tensor-core primitives in inline PTX, for
// kernels that stage their operands in shared memory themselves:
//   * tensor memory (TMEM) allocation by one warp, relinquish, dealloc;
//   * shared-memory matrix descriptors for the no-swizzle K-major layout and
//     the instruction descriptor of tcgen05.mma kind::f16 (BF16 A and B, FP32
//     accumulator in TMEM);
//   * tcgen05.mma issued by one thread, completion signalled by
//     tcgen05.commit on an mbarrier, and a bounded wait on that barrier;
//   * tcgen05.ld of the accumulator (32x32b shape: a warp reads its own
//     quarter of the 128 TMEM lanes, one lane per thread).
//
// Operand layout (no swizzle, K-major): a "core matrix" is 8 rows x 16 bytes
// (8 BF16 values along K), stored contiguously (128 bytes).  The descriptor's
// leading-dimension byte offset (LBO) is the distance between core matrices
// adjacent along K, the stride byte offset (SBO) the distance between core
// matrices adjacent along M (or N).  Tiles here are stored K-block by
// K-block: element (row r, k) of an R-row tile sits at byte
//   ((k / 8) * (R / 8) + r / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so SBO = 128 and LBO = R * 16; one MMA covers K = 16, two core matrices
// along K, and the next K step starts 2 * LBO bytes further.
#pragma once

#include <cstdint>

namespace rskel {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) in an R-row K-major tile (layout above).
__host__ __device__ __forceinline__ uint32_t tile_offset(int r, int k, int R) {
  return (uint32_t)((((k >> 3) * (R >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// --- tensor memory: executed by all 32 lanes of one warp --------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// --- ordering -----------------------------------------------------------------
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Shared-memory writes of this thread become visible to the async proxy
// (the tensor core's operand reads); every writing thread runs it before the
// barrier that precedes the MMA issue.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// --- mbarrier -------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
// Makes a barrier's initialisation visible to the async proxy (the
// tensor core's commit arrives on it); run by the initialising thread.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the barrier's phase `parity` to complete, giving up after
// `max_polls` polls (each try_wait may itself suspend for a while); returns
// false on giving up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// --- descriptors -----------------------------------------------------------------
// Shared-memory matrix descriptor: start address, LBO and SBO (all >> 4),
// the fixed version field 0b001 at bits 46-48, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A (bits 7-9 = 1) and B (bits 10-12 = 1), both K-major, N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// --- MMA --------------------------------------------------------------------------
// D[tmem] (+)= A[adesc] * B[bdesc]^T over K = 16; accumulate = 0 overwrites D.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The mbarrier completes one arrival once every MMA issued before by this
// thread has finished (reading its shared-memory operands included).
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// --- accumulator read-back ----------------------------------------------------------
// Eight consecutive FP32 columns of this thread's TMEM lane (the warp's lane
// quarter must be (warp index % 4)); the wait is inside the same asm so no
// use of the registers can move above it.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r0, r1, r2, r3, r4, r5, r6, r7;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4), "=r"(r5), "=r"(r6), "=r"(r7)
      : "r"(taddr)
      : "memory");
  v[0] = __uint_as_float(r0);
  v[1] = __uint_as_float(r1);
  v[2] = __uint_as_float(r2);
  v[3] = __uint_as_float(r3);
  v[4] = __uint_as_float(r4);
  v[5] = __uint_as_float(r5);
  v[6] = __uint_as_float(r6);
  v[7] = __uint_as_float(r7);
}

}  // namespace tc
}  // namespace rskel
