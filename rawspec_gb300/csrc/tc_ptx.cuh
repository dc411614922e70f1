// tc_ptx.cuh -- inline-PTX wrappers for the 5th-generation tensor cores
// (tcgen05: tensor-memory allocation, MMA issued by one thread, completion
// through an mbarrier, tensor-memory loads) and the shared-memory matrix and
// instruction descriptors they take, after the PTX ISA's tcgen05 chapter.
//
// Conventions used by the kernels:
//  - one CTA (cta_group::1), MMA shape M = 128, K = 16 per instruction,
//    FP16 operands, FP32 accumulator in tensor memory;
//  - both operands K-major without swizzling: a matrix of R rows x K columns
//    is stored as 8-row x 16-byte core matrices; element (r, k) sits at
//    (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2 bytes;
//  - accumulator row r lives in tensor-memory lane r, column j in column j;
//    warp w of the CTA reads lanes [32 (w % 4), 32 (w % 4) + 32).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rsg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices adjacent in K), stride-dimension byte offset
// (between 8-row groups), the fixed 0b001 at bits 46-48, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16 with FP16 A and B, FP32 D, both
// operands K-major, dense: D format at bits 4-5, A/B formats at 7-9 / 10-12
// (0 = F16), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- tensor memory allocation (one whole warp) ----
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- ordering of tensor-core operations around thread synchronisation ----
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes become visible to the tensor cores
// (asynchronous proxy).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- MMA (issued by one thread) ----
// D[tmem] (+)= A[smem] * B[smem]^T, accumulate when acc != 0.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
// The mbarrier receives one arrival when all MMAs issued so far by this
// thread have completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

// ---- operands ----
// Two int8 (re, im) codes of one word -> an FP16 pair, exactly: the bytes
// (offset by 128) become the low mantissa bits of 1024 + v, then 1152 is
// subtracted.  sel picks polarisation 0 (0x4140) or 1 (0x4342).
__device__ __forceinline__ uint32_t codes_to_h2(uint32_t x, uint32_t sel) {
  const uint32_t b = __byte_perm(x, 0x64646464u, sel);
  uint32_t r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(b), "r"(0x64806480u));
  return r;
}

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mb, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}
// One plain arrival (release semantics at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t* mb) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mb)) : "memory");
}
// One arrival that also expects `bytes` of asynchronous copies on the barrier.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)), "r"(bytes) : "memory");
}
// Bulk copy global -> shared (16-byte aligned addresses, size a multiple of
// 16), completing `bytes` transactions on the barrier.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* mb) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(mb))
               : "memory");
}
// Waits for the phase of the given parity, at most `limit` SM clock cycles;
// false on time-out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mb, unsigned parity, long long limit) {
  if (mbar_try_wait(mb, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(mb, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

// ---- tensor memory -> registers ----
// One load of 16 consecutive columns of this thread's lane (32x32b shape),
// then the wait; the registers are tied to the wait so that no use of them
// can be scheduled before it.
__device__ __forceinline__ void tmem_ld16(uint32_t ta, float (&a)[16]) {
  uint32_t* ra = reinterpret_cast<uint32_t*>(a);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(ra[0]), "=r"(ra[1]), "=r"(ra[2]), "=r"(ra[3]), "=r"(ra[4]), "=r"(ra[5]), "=r"(ra[6]), "=r"(ra[7]),
        "=r"(ra[8]), "=r"(ra[9]), "=r"(ra[10]), "=r"(ra[11]), "=r"(ra[12]), "=r"(ra[13]), "=r"(ra[14]),
        "=r"(ra[15])
      : "r"(ta));
  asm volatile(
      "tcgen05.wait::ld.sync.aligned;"
      : "+r"(ra[0]), "+r"(ra[1]), "+r"(ra[2]), "+r"(ra[3]), "+r"(ra[4]), "+r"(ra[5]), "+r"(ra[6]), "+r"(ra[7]),
        "+r"(ra[8]), "+r"(ra[9]), "+r"(ra[10]), "+r"(ra[11]), "+r"(ra[12]), "+r"(ra[13]), "+r"(ra[14]),
        "+r"(ra[15])
      :
      : "memory");
}
// Two loads of 16 consecutive columns of this thread's lane (32x32b shape),
// then the wait; the registers are tied to the wait so that no use of them
// can be scheduled before it.
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float (&a)[16], float (&b)[16]) {
  uint32_t* ra = reinterpret_cast<uint32_t*>(a);
  uint32_t* rb = reinterpret_cast<uint32_t*>(b);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(ra[0]), "=r"(ra[1]), "=r"(ra[2]), "=r"(ra[3]), "=r"(ra[4]), "=r"(ra[5]), "=r"(ra[6]), "=r"(ra[7]),
        "=r"(ra[8]), "=r"(ra[9]), "=r"(ra[10]), "=r"(ra[11]), "=r"(ra[12]), "=r"(ra[13]), "=r"(ra[14]),
        "=r"(ra[15])
      : "r"(ta));
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(rb[0]), "=r"(rb[1]), "=r"(rb[2]), "=r"(rb[3]), "=r"(rb[4]), "=r"(rb[5]), "=r"(rb[6]), "=r"(rb[7]),
        "=r"(rb[8]), "=r"(rb[9]), "=r"(rb[10]), "=r"(rb[11]), "=r"(rb[12]), "=r"(rb[13]), "=r"(rb[14]),
        "=r"(rb[15])
      : "r"(tb));
  asm volatile(
      "tcgen05.wait::ld.sync.aligned;"
      : "+r"(ra[0]), "+r"(ra[1]), "+r"(ra[2]), "+r"(ra[3]), "+r"(ra[4]), "+r"(ra[5]), "+r"(ra[6]), "+r"(ra[7]),
        "+r"(ra[8]), "+r"(ra[9]), "+r"(ra[10]), "+r"(ra[11]), "+r"(ra[12]), "+r"(ra[13]), "+r"(ra[14]),
        "+r"(ra[15]), "+r"(rb[0]), "+r"(rb[1]), "+r"(rb[2]), "+r"(rb[3]), "+r"(rb[4]), "+r"(rb[5]), "+r"(rb[6]),
        "+r"(rb[7]), "+r"(rb[8]), "+r"(rb[9]), "+r"(rb[10]), "+r"(rb[11]), "+r"(rb[12]), "+r"(rb[13]),
        "+r"(rb[14]), "+r"(rb[15])
      :
      : "memory");
}

}  // namespace tc
}  // namespace rsg
