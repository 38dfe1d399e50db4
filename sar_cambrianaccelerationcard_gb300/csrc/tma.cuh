// tma.cuh -- shared-memory mbarriers and bulk (TMA) copies for sm_103a, as
// inline PTX: the staging primitives of the back-projection and the
// persistent range-compression kernels.
#pragma once

#include <cstdint>

namespace sarbp {
namespace {

// limit of each wait for copies still in flight after a wait ran out
constexpr uint64_t kDrainWaitNs = 500000000ull;

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx_arrive(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

// Delivers `bytes` of a phase's expected transaction count without a copy (the
// late bytes of an injected fault).
__device__ __forceinline__ void mbar_complete_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after ~limit_ns and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
#pragma unroll 1
        for (int i = 0; i < 32; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit_ns) return false;
    }
}

// Contiguous global -> shared copy of `bytes` (a multiple of 16, both
// addresses 16-byte aligned) completing on the mbarrier's transaction count.
__device__ __forceinline__ void tma_bulk_g2s(unsigned dst, const void *src, unsigned bytes,
                                             unsigned bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

}  // namespace
}  // namespace sarbp
