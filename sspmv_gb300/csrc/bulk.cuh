// bulk.cuh -- bulk asynchronous copies (the TMA engine's untiled form) from
// global to shared memory, completed on shared-memory mbarriers, for sm_103a.
//
// cp.async.bulk moves a contiguous run of bytes with one instruction issued
// by one thread; the copy engine signals the bytes it delivered on an
// mbarrier (complete_tx), so a CTA can keep several stages of a stream in
// flight while its threads work on an earlier one.  Rules the callers keep:
// global source and shared destination 16-byte aligned, size a multiple of
// 16 bytes, at most 2^20 - 1 bytes per mbarrier phase.
//
// Every wait here is bounded: mbar_wait gives up after kMaxPolls polls and
// returns false, so a kernel never spins forever on a copy that does not
// arrive; the caller records the timeout and leaves in order.
#pragma once

#include <cstdint>

namespace sspmv {

constexpr uint32_t kMaxPolls = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation visible to the copy engine (async proxy).
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory (made
// visible to it by a CTA barrier) before later async-proxy writes: issued
// before a bulk copy overwrites a buffer the CTA has just read or written.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete; false after
// kMaxPolls unsuccessful polls (each poll may itself suspend the thread for
// a short, hardware-defined time).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < kMaxPolls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// bytes from global src to shared dst, completion counted on bar.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace sspmv
