// tc.cuh -- the tcgen05 / TMEM primitives the tensor-core kernels use, as inline
// PTX for sm_103a: TMEM allocation, shared-memory matrix descriptors (K-major,
// no swizzle), single-thread MMA issue, commit to an mbarrier with a bounded
// wait, and TMEM -> register loads.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace dfs {
namespace tc {

DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor for a K-major operand without swizzle: core
// matrices of 8 rows x 16 bytes, `lbo` bytes apart along K and `sbo` bytes apart
// along M/N (both multiples of 16); descriptor version 1 (bits 46-47).
DEV uint64_t desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor: f32 accumulator, K-major A and B, M = 128, N = n.
// fmt = 1 (bf16, kind::f16) or 2 (tf32, kind::tf32).
HD uint32_t idesc(uint32_t fmt, uint32_t n) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

DEV void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

DEV void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

// the same with the A operand in TMEM (row m of A in lane m, two 16-bit elements of K
// per 32-bit column, the lower K in the low half)
DEV void mma_bf16_ts(uint32_t dtmem, uint32_t atmem, uint64_t b, uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}" ::"r"(dtmem),
        "r"(atmem), "l"(b), "r"(id), "r"(accumulate));
}

// arrive on `mbar` when every MMA this thread issued so far has completed
DEV void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)));
}

DEV void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// wait for the phase with parity `phase` to complete, giving up after `limit`
// polls; returns whether it completed
DEV bool mbar_wait(uint64_t* mbar, uint32_t phase, uint32_t limit) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < limit; it++) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase));
        if (done) return true;
    }
    return false;
}

// arrive (release, CTA scope) on `mbar`
DEV void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

DEV void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
DEV void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
DEV void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation by one whole warp; the base address is written to *slot
template <uint32_t COLS>
DEV void tmem_alloc(uint32_t* slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "n"(COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
template <uint32_t COLS>
DEV void tmem_free(uint32_t base) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "n"(COLS));
}

// 16 consecutive f32 columns of this thread's TMEM lane (the warp's 32 lanes)
DEV void ld16(uint32_t taddr, float (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
          "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "r"(taddr));
}
// 8 consecutive f32 columns of this thread's TMEM lane (the warp's 32 lanes); v[8..15] untouched
DEV void ld8(uint32_t taddr, float (&v)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "r"(taddr));
}
DEV void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 consecutive 32-bit columns of this thread's TMEM lane (the warp's 32 lanes) from registers
DEV void st16(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
DEV void st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// packed float pairs (df::pk2 ...) for the epilogues
using df::add2;
using df::fast_two_sum2;
using df::fma2;
using df::mul2;
using df::pk2;
using df::sub2;
using df::two_sum2;
using df::up2;

// byte offset of element (row, k) of a K-major operand with `kgroups` core
// matrices along K per 8-row block (16-byte core rows, `esize`-byte elements)
HD uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t kgroups, uint32_t esize) {
    uint32_t per = 16 / esize;
    return (row / 8) * (128 * kgroups) + (k / per) * 128 + (row % 8) * 16 + (k % per) * esize;
}

}  // namespace tc
}  // namespace dfs
