// tma.cuh -- asynchronous-execution helpers: bulk copies global -> shared (cp.async.bulk)
// completed on mbarriers, and the wait of a programmatically dependent launch.  Bulk copies have
// bounded waits: a wait gives up after TMA_WAIT_NS of the GPU's global timer (or, should the
// timer not advance, after TMA_WAIT_POLLS polls) and returns false, so that a kernel whose
// copy does not arrive can report an error status instead of spinning.
#pragma once

namespace redgb {

constexpr unsigned long long TMA_WAIT_NS = 1000000000ull;  // one second
constexpr unsigned TMA_WAIT_POLLS = 1u << 28;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase)
{
    const unsigned long long t0 = global_ns();
    for (unsigned k = 0; k < TMA_WAIT_POLLS; k++) {
        if (mbar_try_wait(bar, phase)) return true;
        if ((k & 63u) == 63u && global_ns() - t0 > TMA_WAIT_NS) return false;
    }
    return false;
}

// one thread: expect `bytes` on `bar` and start the bulk copy global -> shared
__device__ __forceinline__ void tma_tile(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// one thread: expect `bytes` more on `bar` (the arrival of a barrier initialised with count 1)
__device__ __forceinline__ void mbar_expect(unsigned long long* bar, unsigned bytes)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// one thread: a bulk copy global -> shared completing on `bar` (no arrival of its own);
// both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Programmatic dependent launch: a kernel launched with the programmatic-serialisation
// attribute may be scheduled while the kernel before it on the stream finishes its last CTAs;
// it must not read what that kernel writes before this wait (which returns at once for a
// kernel launched without the attribute).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

}  // namespace redgb
