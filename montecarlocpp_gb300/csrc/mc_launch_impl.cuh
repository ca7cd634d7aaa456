// mc_launch_impl.cuh -- included once per precision translation unit.
#pragma once

#include "mc_launch.h"

namespace mcg {

template <typename K>
static cudaError_t prepare(K fn, size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

// A static-kernel launch; with MC_PDL, programmatic dependent launch: the
// kernel may begin while the previous kernel of the stream finishes (it
// waits for it before touching shared state, griddepcontrol.wait).
template <typename K, typename R>
static cudaError_t launchStatic(K fn, const Params<R>& p, int grid, int threads, size_t smem, cudaStream_t s) {
    if constexpr (MC_PDL != 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, fn, p);
    } else {
        fn<<<grid, threads, smem, s>>>(p);
        return cudaGetLastError();
    }
}

// GEN: the kernels that also take subdomains other than the Parallelepiped,
// continuation slots and Inter faces paired more than once.
template <typename R, bool DYN, bool REPLAY, bool LOG, int TM, bool GEN = false>
static cudaError_t advanceOne(const Params<R>& p, int grid, int block, size_t smem, cudaStream_t s) {
    auto fn = DYN ? k_advance_dyn<R, REPLAY, LOG, TM, GEN> : k_advance<R, REPLAY, LOG, TM, -1, GEN>;
    cudaError_t e = prepare(fn, smem);
    if (e != cudaSuccess) return e;
    // the static kernel adds its producer warp to the `block` consumers
    if (!DYN) return launchStatic(fn, p, grid, block + STATIC_PRODUCER_THREADS, smem, s);
    fn<<<grid, block, smem, s>>>(p);
    return cudaGetLastError();
}

template <typename R, bool DYN, bool REPLAY, bool LOG, int TM, bool GEN = false>
static int occOne(int block, size_t smem) {
    auto fn = DYN ? k_advance_dyn<R, REPLAY, LOG, TM, GEN> : k_advance<R, REPLAY, LOG, TM, -1, GEN>;
    if (prepare(fn, smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, DYN ? block : block + STATIC_PRODUCER_THREADS, smem) !=
        cudaSuccess)
        return 0;
    return nb;
}

// The static kernel with the lean flight along axis `lean` (0..2).
template <>
cudaError_t launchAdvanceLean<MC_REAL>(const Params<MC_REAL>& p, int lean, int grid, int block, size_t smem,
                                       cudaStream_t s) {
    auto fn = lean == 0 ? k_advance<MC_REAL, false, false, TM_SHARED, 0>
            : lean == 1 ? k_advance<MC_REAL, false, false, TM_SHARED, 1>
                        : k_advance<MC_REAL, false, false, TM_SHARED, 2>;
    cudaError_t e = prepare(fn, smem);
    if (e != cudaSuccess) return e;
    return launchStatic(fn, p, grid, block + STATIC_PRODUCER_THREADS, smem, s);
}

template <>
int advanceLeanOccupancy<MC_REAL>(int lean, int block, size_t smem) {
    auto fn = lean == 0 ? k_advance<MC_REAL, false, false, TM_SHARED, 0>
            : lean == 1 ? k_advance<MC_REAL, false, false, TM_SHARED, 1>
                        : k_advance<MC_REAL, false, false, TM_SHARED, 2>;
    if (prepare(fn, smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block + STATIC_PRODUCER_THREADS, smem) != cudaSuccess)
        return 0;
    return nb;
}

template <>
cudaError_t launchEmit<MC_REAL>(const Params<MC_REAL>& p, bool replay, cudaStream_t s) {
    if (p.nemit <= 0) return cudaSuccess;
    int block = 256;
    long long grid = (p.nemit + block - 1) / block;
    if (replay) k_emit<MC_REAL, true><<<(unsigned)grid, block, 0, s>>>(p);
    else k_emit<MC_REAL, false><<<(unsigned)grid, block, 0, s>>>(p);
    return cudaGetLastError();
}

template <>
cudaError_t launchCompact<MC_REAL>(const Params<MC_REAL>& p, int grid, cudaStream_t s) {
    k_compact<MC_REAL><<<grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

template <>
cudaError_t launchEmitBatch<MC_REAL>(const Params<MC_REAL>& p, cudaStream_t s) {
    if (p.cap == 0) return cudaSuccess;
    const long long grid = ((long long)p.cap + 255) / 256;
    k_emit_batch<MC_REAL><<<(unsigned)grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
static auto batchKernel(int tm, bool gen) {
    if (gen) return k_advance_batch<R, TM_AUTO, true>;
    return tm == TM_SHARED ? k_advance_batch<R, TM_SHARED>
         : tm == TM_GLOBAL ? k_advance_batch<R, TM_GLOBAL>
         : tm == TM_NONE   ? k_advance_batch<R, TM_NONE>
                           : k_advance_batch<R, TM_AUTO>;
}

template <>
cudaError_t launchAdvanceBatch<MC_REAL>(const Params<MC_REAL>& p, int tm, bool gen, int grid, int block,
                                        cudaStream_t s) {
    const size_t smem = batchSmemBytes<MC_REAL>(p);
    auto fn = batchKernel<MC_REAL>(tm, gen);
    cudaError_t e = prepare(fn, smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, s>>>(p);
    return cudaGetLastError();
}

template <>
cudaError_t launchDifPrefix<MC_REAL>(const Params<MC_REAL>& p, cudaStream_t s) {
    k_difprefix<MC_REAL><<<dim3((unsigned)p.ninst, (unsigned)p.maxRows * (unsigned)p.maxGroups), 32, 0, s>>>(p);
    return cudaGetLastError();
}

template <>
cudaError_t launchRoundReduce<MC_REAL>(const Params<MC_REAL>& p, double* const* accs, double* gsum,
                                       cudaStream_t s) {
    k_round_reduce<MC_REAL><<<dim3(64, (unsigned)p.ninst), 256, 0, s>>>(p, accs, gsum);
    return cudaGetLastError();
}

template <>
int advanceBatchOccupancy<MC_REAL>(int tm, bool gen, size_t smem, int block) {
    auto fn = batchKernel<MC_REAL>(tm, gen);
    if (prepare(fn, smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, smem) != cudaSuccess) return 0;
    return nb;
}

#define MC_DISPATCH(F, ...)                                                                 \
    if (gen && replay) {                                                                   \
        if (dyn) {                                                                         \
            if (tm == TM_SHARED) return log ? F<MC_REAL, true, true, true, TM_SHARED, true>(__VA_ARGS__)   \
                                            : F<MC_REAL, true, true, false, TM_SHARED, true>(__VA_ARGS__);  \
            return log ? F<MC_REAL, true, true, true, TM_GLOBAL, true>(__VA_ARGS__)           \
                       : F<MC_REAL, true, true, false, TM_GLOBAL, true>(__VA_ARGS__);         \
        }                                                                                  \
        if (tm == TM_SHARED) return log ? F<MC_REAL, false, true, true, TM_SHARED, true>(__VA_ARGS__)      \
                                        : F<MC_REAL, false, true, false, TM_SHARED, true>(__VA_ARGS__);     \
        return log ? F<MC_REAL, false, true, true, TM_GLOBAL, true>(__VA_ARGS__)              \
                   : F<MC_REAL, false, true, false, TM_GLOBAL, true>(__VA_ARGS__);            \
    }                                                                                      \
    if (gen) {                                                                             \
        if (dyn) {                                                                         \
            if (tm == TM_SHARED) return log ? F<MC_REAL, true, false, true, TM_SHARED, true>(__VA_ARGS__)  \
                                            : F<MC_REAL, true, false, false, TM_SHARED, true>(__VA_ARGS__); \
            return log ? F<MC_REAL, true, false, true, TM_GLOBAL, true>(__VA_ARGS__)          \
                       : F<MC_REAL, true, false, false, TM_GLOBAL, true>(__VA_ARGS__);        \
        }                                                                                  \
        if (tm == TM_SHARED) return log ? F<MC_REAL, false, false, true, TM_SHARED, true>(__VA_ARGS__)     \
                                        : F<MC_REAL, false, false, false, TM_SHARED, true>(__VA_ARGS__);    \
        return log ? F<MC_REAL, false, false, true, TM_GLOBAL, true>(__VA_ARGS__)             \
                   : F<MC_REAL, false, false, false, TM_GLOBAL, true>(__VA_ARGS__);           \
    }                                                                                      \
    if (dyn) {                                                                             \
        if (tm == TM_SHARED) {                                                             \
            if (replay) return log ? F<MC_REAL, true, true, true, TM_SHARED>(__VA_ARGS__)   \
                                   : F<MC_REAL, true, true, false, TM_SHARED>(__VA_ARGS__); \
            return log ? F<MC_REAL, true, false, true, TM_SHARED>(__VA_ARGS__)              \
                       : F<MC_REAL, true, false, false, TM_SHARED>(__VA_ARGS__);            \
        }                                                                                  \
        if (replay) return log ? F<MC_REAL, true, true, true, TM_GLOBAL>(__VA_ARGS__)       \
                               : F<MC_REAL, true, true, false, TM_GLOBAL>(__VA_ARGS__);     \
        return log ? F<MC_REAL, true, false, true, TM_GLOBAL>(__VA_ARGS__)                  \
                   : F<MC_REAL, true, false, false, TM_GLOBAL>(__VA_ARGS__);                \
    }                                                                                      \
    if (tm == TM_SHARED) {                                                                 \
        if (replay) return log ? F<MC_REAL, false, true, true, TM_SHARED>(__VA_ARGS__)      \
                               : F<MC_REAL, false, true, false, TM_SHARED>(__VA_ARGS__);    \
        return log ? F<MC_REAL, false, false, true, TM_SHARED>(__VA_ARGS__)                 \
                   : F<MC_REAL, false, false, false, TM_SHARED>(__VA_ARGS__);               \
    }                                                                                      \
    if (replay) return log ? F<MC_REAL, false, true, true, TM_GLOBAL>(__VA_ARGS__)          \
                           : F<MC_REAL, false, true, false, TM_GLOBAL>(__VA_ARGS__);        \
    return log ? F<MC_REAL, false, false, true, TM_GLOBAL>(__VA_ARGS__)                     \
               : F<MC_REAL, false, false, false, TM_GLOBAL>(__VA_ARGS__);

template <>
cudaError_t launchAdvance<MC_REAL>(const Params<MC_REAL>& p, bool dyn, bool replay, bool log, int tm, bool gen,
                                   int grid, int block, size_t smem, cudaStream_t s) {
    MC_DISPATCH(advanceOne, p, grid, block, smem, s)
}

template <>
int advanceOccupancy<MC_REAL>(bool dyn, bool replay, bool log, int tm, bool gen, int block, size_t smem) {
    MC_DISPATCH(occOne, block, smem)
}

#undef MC_DISPATCH

}  // namespace mcg
