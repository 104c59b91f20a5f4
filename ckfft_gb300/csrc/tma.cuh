// tma.cuh -- bulk-copy (TMA) and mbarrier helpers, inline PTX for sm_90+ / sm_103a.
//
// Only the 1-D bulk form is used (cp.async.bulk global -> shared with an
// mbarrier completing on the transferred byte count): frames of a batch are
// contiguous, so one copy moves a whole group of frames.  Copies need 16-byte
// aligned addresses and a byte count that is a multiple of 16; callers check.
//
// Every wait is bounded.  A wait that runs out records kErrWaitTimeout in the
// error word the kernel was given and returns false; kernels then stop.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ckg {

constexpr unsigned kErrWaitTimeout = 1u;
constexpr int kWaitTries = 1 << 22;   // each try suspends briefly; bounded to seconds

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) accesses to the same memory.
__device__ __forceinline__ void fence_proxy_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(bar), "r"(phase) : "memory");
    return ok != 0;
}

// Waits for `phase` of the barrier; false (and the error word set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, unsigned* err, int tries = kWaitTries)
{
#pragma unroll 1
    for (int it = 0; it < tries; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    if (err) *(volatile unsigned*)err = kErrWaitTimeout;   // plain store: err may be host-mapped
    return false;
}

}  // namespace ckg
