/*
 * tma.cuh - inline-PTX helpers for bulk asynchronous copies (TMA, 1-D
 * cp.async.bulk) tracked by shared-memory mbarriers, sm_90+ / sm_103a.
 *
 * Every wait is bounded by the global nanosecond timer: a wait that runs out
 * records an error code in *err and returns false, so a kernel never spins
 * forever on a copy that does not arrive.
 */
#ifndef UFOIR_TMA_CUH
#define UFOIR_TMA_CUH

#include <cstdint>

namespace tma {

/* Error codes written to the kernel error word. */
enum : int { kErrWaitTimeout = 1, kErrDrainTimeout = 2, kErrWindow = 8 };

constexpr unsigned long long kWaitLimitNs = 250000000ull;   /* 250 ms */

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

/* Makes barrier initialisation visible to the async proxy. */
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

/* Orders this thread's earlier generic-proxy shared-memory accesses before
 * later async-proxy (bulk copy) accesses. */
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

/* 1-D bulk copy global -> shared; dst, src 16-byte aligned, bytes % 16 == 0. */
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

/* Wait for phase `parity` of the barrier; false (and *err set) after the limit. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, int code)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > kWaitLimitNs) {
            if (err)
                atomicExch(err, code);
            return false;
        }
    }
    return true;
}

}  // namespace tma

#endif
