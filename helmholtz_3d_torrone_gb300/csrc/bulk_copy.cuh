// bulk_copy.cuh -- 1-D TMA bulk copies (cp.async.bulk) into shared memory,
// completed on an mbarrier, with bounded waits.
//
// Rules kept by every caller: global source and shared destination are
// 16-byte aligned and every copy size is a multiple of 16 bytes.  Every wait
// polls a bounded number of times; on timeout it reports failure instead of
// spinning forever, so a lost copy turns into an error status, not a hang.
#pragma once

#include <cstdint>

namespace hz {

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
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

// Bounded wait for the given phase parity; returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, long long limit)
{
    for (long long i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Poll limit of the data waits (a CTA waiting for its next source tile).
// Each translation unit that includes this header holds its own copy on
// every device; hz_set_wait_limit sets them all on the current device (a
// short limit makes the waits give up, for tests of the error path).
static __device__ long long g_data_wait_limit = 1ll << 24;

// After a data wait gave up: the copies this CTA still has in flight (the
// buffer waited on and, when it was issued, the other one) must land before
// the CTA exits and its shared memory is reused.  Called by the thread that
// issued them; these waits keep the full bound whatever the data-wait limit.
__device__ __forceinline__ void mbar_drain(uint64_t *cur, uint32_t pcur, uint64_t *other, uint32_t pother,
                                           bool other_issued)
{
    mbar_wait_bounded(cur, pcur, 1ll << 24);
    if (other_issued) mbar_wait_bounded(other, pother, 1ll << 24);
}

// Host side: set this translation unit's copy of the limit on the current device.
#define HZ_DEFINE_WAIT_LIMIT_SETTER(name)                                                        \
    int name(long long polls)                                                                    \
    {                                                                                            \
        return cudaMemcpyToSymbol(g_data_wait_limit, &polls, sizeof(polls)) == cudaSuccess ? 0 : -1; \
    }

}  // namespace hz
