// tma.cuh -- bulk-copy (TMA) and mbarrier helpers shared by the kernels that
// stage their inputs in shared memory (inline PTX, sm_90+ forms).
#pragma once
#include <stdint.h>

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// one contiguous bulk copy global -> shared (both 16-byte aligned, bytes a
// multiple of 16), completing on the mbarrier
__device__ __forceinline__ void tma_load(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// bounded wait: returns false (and the caller reports an error) if the
// barrier phase does not complete within the iteration limit
#define MBAR_POLLS (1LL << 24)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, long long polls = MBAR_POLLS)
{
    const unsigned a = smem_u32(bar);
    for (long long it = 0; it < polls; it++) {
        unsigned ok;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}
