// Device helpers shared by the split-precision product kernels: mbarriers,
// bulk copies, tcgen05 MMA / TMEM access and the 128-byte-swizzled K-major
// operand layout (inline PTX for sm_103a).
#pragma once
#include <cstdint>

#include "ozaki.cuh"

namespace nvpt {
namespace oz {

constexpr uint32_t kSpinLimit = 1u << 22;  // polls (with ~100 ns back-off) before a wait gives up

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\tselp.u32 %0, 1, 0, P;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on the phase with the given parity.  Gives up (returning
// false) when the limit is reached -- setting *err -- or when another role
// has already set *err.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int *err) {
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
        if (mbar_test(bar, parity)) return true;
        if ((i & 255u) == 255u && *(volatile int *)err) return false;
        if (i > 1024) __nanosleep(100);
    }
    atomicExch(err, 1);
    return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// UMMA shared-memory descriptor, K-major with the 128-byte swizzle (start,
// leading-dim offset unused, stride offset = next 8-row group, version 1,
// layout type 2).  The start may sit at a 32-byte K step inside a 1024-byte
// aligned swizzle atom.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)((SBO_SW >> 4) & 0x3FFFu) << 32) |
           (1ull << 46) | (2ull << 61);
}
// Byte offset of element (r, k) (k < KC) in a swizzled K-major tile.
__host__ __device__ __forceinline__ uint32_t sw128_off(int r, int k) {
    return (uint32_t)(r * ROWB + ((((k >> 3) ^ r) & 7) << 4) + (k & 7) * 2);
}

// Instruction descriptor: D f32, A bf16, B bf16, both K-major, M = 128.
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 2^e as a double (normal range).
__device__ __forceinline__ double pow2(int e) {
    e = max(-1022, min(1023, e));
    return __longlong_as_double((long long)(e + 1023) << 52);
}

__device__ __forceinline__ int exp_above(double m) {  // smallest E with m < 2^E (m >= 0)
    if (!(m > 0.0)) return 0;
    int e;
    frexp(m, &e);
    return e;
}

}  // namespace oz
}  // namespace nvpt
