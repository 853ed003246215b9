// Bulk global->shared copies (cp.async.bulk, the TMA's 1D form) completed on a
// shared-memory mbarrier, for kernels that stream contiguous particle arrays
// through shared memory in double-buffered batches.
//
// Rules the callers keep: source and destination 16-byte aligned, sizes a
// multiple of 16 bytes; one thread initialises the barriers and issues each
// copy; waits have an iteration limit, and either one thread waits and
// publishes the outcome through shared memory or every thread waits for itself
// and the CTA agrees on the outcome at its next barrier, so that the whole CTA
// proceeds or leaves together.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pyl {

// A bounded wait gives up after this many SM clock cycles (about 0.1 s), or as
// soon as another CTA has reported a failed wait.
constexpr long long MBAR_WAIT_CYCLES = 200000000LL;

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the asynchronous (copy) proxy.
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of `bar`; false (and *err set) when the time
// limit runs out or *err is already set.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity, unsigned *err,
                                                  long long limit = MBAR_WAIT_CYCLES)
{
    const long long t0 = clock64();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > limit || *(volatile unsigned *)err) break;
    }
    atomicOr(err, 1u);
    return false;
}

// Waits for phase `parity` of `bar` for at most MBAR_WAIT_CYCLES whatever the
// error word says: the drain of a CTA's own copies after a failed wait.
__device__ __forceinline__ bool mbar_drain_bounded(unsigned long long *bar, unsigned parity)
{
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > MBAR_WAIT_CYCLES) return false;
    return true;
}

// Orders this thread's (and, after a barrier, the CTA's) generic-proxy accesses
// of shared memory before later bulk copies into it.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Issues one bulk copy of `bytes` (multiple of 16, may be 0) into dst, arming
// `bar` for it.  Called by one thread.
__device__ __forceinline__ void stage_copy(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    mbar_arrive_expect_tx(bar, bytes);
    if (bytes) bulk_g2s(dst, src, bytes, bar);
}

}  // namespace pyl
