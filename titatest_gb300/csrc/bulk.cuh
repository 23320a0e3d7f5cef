// Bulk asynchronous copies (cp.async.bulk, the TMA engine's untiled form)
// completing on shared-memory mbarriers, sm_90+.
//
// Rules kept by every caller: source and destination 16-byte aligned, sizes
// a multiple of 16 bytes, at most 2^20 - 1 bytes in flight per barrier phase.
// Every wait is bounded: mbar_wait() gives up after kSpinLimit polls (each
// poll is a hardware try_wait that itself suspends for a bounded time) and
// returns false, and the caller reports a device error instead of hanging.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace crgpu {

constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// order this thread's earlier generic shared-memory accesses before later
// async-proxy (bulk copy) writes to the same buffers
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// global -> shared bulk copy signalling `bar` with the transferred bytes
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
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

// wait for the completion of the barrier phase with the given parity;
// false after kSpinLimit polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (int it = 0; it < kSpinLimit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s: far above any legitimate wait

// try_wait that lets the thread sleep (up to `ns`) until the phase completes,
// so waiting warps leave the issue slots to the warps doing the work
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity, uint32_t ns) {
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}

// mbar_wait for kernels whose roles wait on one another: gives up when
// another thread has raised *abort, or after kWaitNs (then raises it).
// sleep_ns > 0 lets the waiting thread sleep between polls (for waits off
// the critical path); 0 polls without sleeping.
__device__ __forceinline__ bool mbar_wait_abort(uint64_t *bar, uint32_t parity, volatile int *abort,
                                                uint32_t sleep_ns = 20000u) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t it = 1;; it++) {
        if (sleep_ns ? mbar_try_wait_sleep(bar, parity, sleep_ns) : mbar_try_wait(bar, parity)) return true;
        if ((it & 15u) == 0u) {
            if (*abort) return false;
            if (globaltimer_ns() - t0 > kWaitNs) {
                *abort = 1;
                return false;
            }
        }
    }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

}  // namespace crgpu
