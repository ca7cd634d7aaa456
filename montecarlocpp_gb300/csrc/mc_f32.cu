// FP32 flight kernels (FP64 tallies).
#define MC_REAL float
#include "mc_launch_impl.cuh"

namespace mcg {

// Self-check of the bounded waits: one thread waits for a phase of an
// mbarrier that nothing completes, with a deadline of limitNs. The wait must
// give up (S_TIMEOUT) after about that long; the thread then completes the
// phase itself, so nothing is left pending when the block exits.
__global__ void __launch_bounds__(32) k_wait_check(unsigned* status, unsigned long long limitNs,
                                                   unsigned long long* waitedNs) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbarInit(&bar, 1);
        mbarInitFence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint64_t t0 = globalTimerNs();
        const bool done = mbarWait(&bar, 0u, limitNs);
        *waitedNs = globalTimerNs() - t0;
        if (!done) atomicOr(status, (unsigned)S_TIMEOUT);
        mbarArrive(&bar);
    }
}

cudaError_t launchWaitCheck(unsigned* status, unsigned long long limitNs, unsigned long long* waitedNs,
                            cudaStream_t s) {
    k_wait_check<<<1, 32, 0, s>>>(status, limitNs, waitedNs);
    return cudaGetLastError();
}

}  // namespace mcg
