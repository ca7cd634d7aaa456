// mc_launch.h -- host-side launch wrappers of the sm_103a kernels, one
// instantiation per precision (mc_f32.cu, mc_f64.cu).
#pragma once

#include <cuda_runtime.h>

#include "mc_kernels.cuh"

namespace mcg {

template <typename R>
cudaError_t launchEmit(const Params<R>& p, bool replay, cudaStream_t s);

// tm: TM_SHARED or TM_GLOBAL; dyn: the dynamic-refill kernel
template <typename R>
cudaError_t launchAdvance(const Params<R>& p, bool dyn, bool replay, bool log, int tm, bool gen, int grid,
                          int block, size_t smem, cudaStream_t s);

template <typename R>
cudaError_t launchCompact(const Params<R>& p, int grid, cudaStream_t s);

// static kernel with the lean flight of a 1-D shared field along axis lean
template <typename R>
cudaError_t launchAdvanceLean(const Params<R>& p, int lean, int grid, int block, size_t smem, cudaStream_t s);
template <typename R>
int advanceLeanOccupancy(int lean, int block, size_t smem);

// batched launches (all instances in one kernel)
template <typename R>
cudaError_t launchEmitBatch(const Params<R>& p, cudaStream_t s);
// tm: the launch's common field mode (TM_SHARED / TM_GLOBAL / TM_NONE) or
// TM_AUTO (batchFieldMode)
template <typename R>
cudaError_t launchAdvanceBatch(const Params<R>& p, int tm, bool gen, int grid, int block, cudaStream_t s);
template <typename R>
cudaError_t launchDifPrefix(const Params<R>& p, cudaStream_t s);
template <typename R>
int advanceBatchOccupancy(int tm, bool gen, size_t smem, int block);
template <typename R>
cudaError_t launchRoundReduce(const Params<R>& p, double* const* accs, double* gsum,
                              cudaStream_t s);

// device build of the temperature-dependent Material tables of n
// temperatures (mc_material_create_many); all arrays device memory, per
// temperature t at offset t * (nw, nw * np, 4) of each output
struct MatBuildArgs {
    long nw, np;
    const double *omega, *domega, *vel, *dos, *relax, *T;
    double* tau;
    double* sums;     // energySum, fluxSum, scatSum, cond
    unsigned long long *swthr, *spthr, *fwthr, *fpthr;
    double* scratch;  // 3 nw np per temperature
    double* rows;     // 2 nw per temperature
    int* status;      // 1: a non-finite relaxation time or a zero velocity
};
cudaError_t launchBuildMaterials(const MatBuildArgs& a, int n, cudaStream_t s);

// the bounded-wait self-check (mc_check_bounded_wait)
cudaError_t launchWaitCheck(unsigned* status, unsigned long long limitNs, unsigned long long* waitedNs,
                            cudaStream_t s);

// Maximum resident blocks per SM of the advance kernel for this
// configuration (0 if it cannot launch).
template <typename R>
int advanceOccupancy(bool dyn, bool replay, bool log, int tm, bool gen, int block, size_t smem);

}  // namespace mcg
