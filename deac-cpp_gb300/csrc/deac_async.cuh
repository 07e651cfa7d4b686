// deac_async.cuh -- shared-memory barriers and bulk copies (sm_90 and later
// PTX), used by the split engine's kernels.  Every wait is bounded: it gives
// up after kWaitNs of wall time and the caller reports an error status.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace deac {

constexpr uint64_t kWaitNs = 2000000000ull;  // bounded mbarrier waits: 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// an mbarrier expecting `count` arrivals per phase; the initialisation is
// made visible to the asynchronous proxy (bulk copies) as well
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// more bytes to come in the current phase, without an arrival
__device__ __forceinline__ void mbar_add_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// whether the phase with parity `phase` has completed, the thread suspended
// in the meantime (woken when the phase completes, or after a time limit
// of the hardware's choosing)
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t phase) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return done != 0;
}

// Wait for the completion of the mbarrier phase with parity `phase`, giving
// up after kWaitNs of wall time (the caller then reports an error).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    if (mbar_try(bar, phase)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try(bar, phase)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

// One bulk copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) from global to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace deac
