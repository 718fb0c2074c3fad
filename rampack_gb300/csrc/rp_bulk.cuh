// Bulk asynchronous copies global -> shared memory (cp.async.bulk: the TMA engine's untiled
// form) completing on a shared-memory mbarrier, and a bounded wait on that barrier.
//
// Rules the callers keep: both addresses 16-byte aligned and the size a multiple of 16; the
// expected byte count of a phase registered (arrive.expect_tx) before the phase's copies are
// waited for; generic-proxy accesses of a buffer ordered before the async proxy overwrites it
// (fence_proxy_async_smem by every accessing thread, then a barrier, then the copies).
#pragma once

#include <cstdint>

namespace rp {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// A barrier expecting `count` arrivals per phase, starting in phase 0.
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the async proxy (the copies' completion).
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Orders this thread's earlier generic-proxy accesses of shared memory before later
// async-proxy accesses (a bulk copy overwriting what the thread read or wrote).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One arrival on the barrier, registering `bytes` more to arrive by copies in this phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// `bytes` from global `src` to shared `dst`, counted on `bar` when they have landed.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Whether the phase of the given parity has completed (non-blocking).
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of the given parity; false after `limit` polls (about 40 ns apart).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int limit) {
    for (int i = 0; i < limit; i++) {
        if (mbar_test(bar, parity)) return true;
        __nanosleep(32);
    }
    return false;
}

}  // namespace rp
