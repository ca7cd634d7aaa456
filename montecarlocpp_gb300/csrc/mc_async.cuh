// mc_async.cuh -- sm_90+/sm_103a asynchronous-copy building blocks in inline
// PTX: mbarriers, one-dimensional bulk copies (cp.async.bulk, the TMA engine
// without a tensor map) from global into shared memory, and a named
// barrier with an OR reduction.
//
// Every wait is bounded: it polls mbarrier.try_wait until the phase
// completes or a deadline on %globaltimer passes, and reports which. A
// caller that gives up sets an error status and stops issuing work, so no
// kernel built on these helpers can spin forever.
#pragma once

#include <stdint.h>

namespace mcg {

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globalTimerNs() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async proxy (bulk copies)
// before any thread uses the barriers; a block barrier must follow.
__device__ __forceinline__ void mbarInitFence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbarArrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smemAddr(bar))
                 : "memory");
}

// Arrive and add `bytes` to the transaction count the phase waits for.
__device__ __forceinline__ void mbarArriveExpectTx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smemAddr(bar)),
                 "r"(bytes)
                 : "memory");
}

// One try: the thread may be suspended (not spinning on issue slots) until
// the phase completes or about `hintNs` nanoseconds have passed.
__device__ __forceinline__ bool mbarTryWait(uint64_t* bar, uint32_t parity, uint32_t hintNs = 100000u) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(bar)), "r"(parity), "r"(hintNs)
        : "memory");
    return ok != 0;
}

// Wait for the phase of parity `parity` to complete; false once `limitNs`
// nanoseconds have passed (the phase may still complete later) or when
// *stop becomes non-zero (another role of the block gave up). Each try
// suspends the thread for up to 100 us, so a waiting warp leaves the issue
// slots to the warps that are working.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity, uint64_t limitNs,
                                         const volatile int* stop = nullptr) {
    if (mbarTryWait(bar, parity)) return true;
    const uint64_t t0 = globalTimerNs();
    for (;;) {
        if (mbarTryWait(bar, parity)) return true;
        if (stop != nullptr && *stop) return false;
        if (globalTimerNs() - t0 > limitNs) return false;
    }
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global memory into this block's shared memory; completion is
// signalled as transaction bytes on `bar`.
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smemAddr(dst)),
        "l"(src), "r"(bytes), "r"(smemAddr(bar))
        : "memory");
}

// Programmatic dependent launch (sm_90+). A kernel launched with the
// programmatic stream-serialization attribute may start while the kernel
// before it in the stream is still running; gridDepWait blocks until that
// kernel has completed and its memory writes are visible (a no-op without
// such a predecessor), gridDepTrigger lets the next such kernel be scheduled
// as this one's blocks exit.
__device__ __forceinline__ void gridDepWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void gridDepTrigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Named barrier `id` over `nthreads` threads (a multiple of 32) that also
// returns the OR of `pred` over them: every participant gets the same answer.
__device__ __forceinline__ bool barOr(int id, int nthreads, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id), "r"(nthreads)
        : "memory");
    return r != 0;
}

}  // namespace mcg
