// bulk.cuh -- bulk asynchronous copies (the TMA engine's untiled form,
// cp.async.bulk) from global into shared memory, completed on an mbarrier.
//
// A copy needs 16-byte aligned source and destination and a size that is a
// multiple of 16 bytes.  Waits are bounded in time: a wait that has not seen its
// phase complete after one second returns false, and the caller records an
// error and drains its copies instead of spinning on.
#pragma once
#include <stdint.h>

namespace amk {
namespace bulk {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void bar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival that also announces `bytes` of copies completing on this phase
__device__ __forceinline__ void bar_expect(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void copy_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// one plain arrival (release: this thread's earlier shared-memory accesses are
// ordered before the phase completes)
__device__ __forceinline__ void bar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// orders this thread's earlier shared-memory accesses before later copies into them
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool bar_try(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{ .reg .pred P; mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2; selp.u32 %0, 1, 0, P; }"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// waits for phase `parity` of `bar`; false after `limit_ns` (one second) without it
__device__ __forceinline__ bool bar_wait(uint64_t *bar, unsigned parity,
                                         unsigned long long limit_ns = 1000000000ull) {
    if (bar_try(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!bar_try(bar, parity))
        if (now_ns() - t0 > limit_ns) return false;
    return true;
}

}  // namespace bulk
}  // namespace amk
