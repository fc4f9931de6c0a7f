// tde_tc.cuh -- 5th-generation tensor core (tcgen05) primitives for sm_103a,
// written as inline PTX: shared-memory matrix descriptors, the bf16 MMA with
// an FP32 accumulator in tensor memory (TMEM), TMEM allocation and loads,
// and bounded mbarrier waits.
//
// Operand layouts used here have no swizzle.  A "core matrix" is 8 rows of 16
// contiguous bytes, 128 bytes in all: for a K-major operand each row holds 8
// bf16 along K, for an MN-major operand 8 bf16 along M (or N) of one k.  A
// descriptor names the first core matrix and two strides, in both cases:
//   LBO -- bytes between core matrices adjacent along K,
//   SBO -- bytes between core matrices adjacent along M (or N).
// One kind::f16 MMA consumes K = 16 (two core matrices along K).
#pragma once

#include <stdint.h>

namespace tde {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start, LBO and SBO in 16-byte units,
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63).
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16;
    d |= static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// bf16 A (bits 7-9 = 1) and B (bits 10-12 = 1), both K-major (bits 15, 16 =
// 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// The mbarrier completes one phase when every MMA this thread issued so far
// has finished (and its shared-memory reads with it).
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Makes this thread's ordinary shared-memory stores visible to the tensor
// core (the async proxy); used before the barrier that precedes the MMA.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// TMEM allocation: executed by one whole warp; the base address is written
// to *slot.  ncols is a power of two in [32, 512].
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Warp-collective: lane i receives 16 consecutive 32-bit columns of TMEM
// lane (lane base + i), starting at the column of taddr.  A warp may only
// read the 32 lanes of its quarter (warp index % 4).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// mbarrier
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// As mbar_try_wait, letting the thread sleep up to `hint_ns` nanoseconds for
// the phase to complete instead of returning at once.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *b, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase with the given parity to complete, for at most
// `limit_ns` nanoseconds; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, uint64_t limit_ns = 2000000000ull) {
    if (mbar_try_wait(b, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(b, parity))
        if (globaltimer_ns() - t0 > limit_ns) return false;
    return true;
}

}  // namespace tc
}  // namespace tde
