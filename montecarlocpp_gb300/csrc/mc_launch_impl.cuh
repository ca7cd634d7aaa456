// mc_launch_impl.cuh -- included once per precision translation unit.
#pragma once

#include "mc_launch.h"

namespace mcg {

template <typename R, bool REPLAY, bool LOG, int TM>
static cudaError_t advanceOne(const Params<R>& p, int grid, int block, size_t smem, cudaStream_t s) {
    auto fn = k_advance<R, REPLAY, LOG, TM>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, s>>>(p);
    return cudaGetLastError();
}

template <typename R, bool REPLAY, bool LOG, int TM>
static int occOne(int block, size_t smem) {
    auto fn = k_advance<R, REPLAY, LOG, TM>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, smem) != cudaSuccess) return 0;
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
cudaError_t launchAdvance<MC_REAL>(const Params<MC_REAL>& p, bool replay, bool log, int tm, int grid,
                                   int block, size_t smem, cudaStream_t s) {
    if (tm == TM_SHARED) {
        if (replay) return log ? advanceOne<MC_REAL, true, true, TM_SHARED>(p, grid, block, smem, s)
                               : advanceOne<MC_REAL, true, false, TM_SHARED>(p, grid, block, smem, s);
        return log ? advanceOne<MC_REAL, false, true, TM_SHARED>(p, grid, block, smem, s)
                   : advanceOne<MC_REAL, false, false, TM_SHARED>(p, grid, block, smem, s);
    }
    if (replay) return log ? advanceOne<MC_REAL, true, true, TM_GLOBAL>(p, grid, block, smem, s)
                           : advanceOne<MC_REAL, true, false, TM_GLOBAL>(p, grid, block, smem, s);
    return log ? advanceOne<MC_REAL, false, true, TM_GLOBAL>(p, grid, block, smem, s)
               : advanceOne<MC_REAL, false, false, TM_GLOBAL>(p, grid, block, smem, s);
}

template <>
int advanceOccupancy<MC_REAL>(bool replay, bool log, int tm, int block, size_t smem) {
    if (tm == TM_SHARED) {
        if (replay) return log ? occOne<MC_REAL, true, true, TM_SHARED>(block, smem)
                               : occOne<MC_REAL, true, false, TM_SHARED>(block, smem);
        return log ? occOne<MC_REAL, false, true, TM_SHARED>(block, smem)
                   : occOne<MC_REAL, false, false, TM_SHARED>(block, smem);
    }
    if (replay) return log ? occOne<MC_REAL, true, true, TM_GLOBAL>(block, smem)
                           : occOne<MC_REAL, true, false, TM_GLOBAL>(block, smem);
    return log ? occOne<MC_REAL, false, true, TM_GLOBAL>(block, smem)
               : occOne<MC_REAL, false, false, TM_GLOBAL>(block, smem);
}

}  // namespace mcg
