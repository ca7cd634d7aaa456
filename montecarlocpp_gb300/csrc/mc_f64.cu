// FP64 flight kernels; built with --fmad=false so that products and sums
// round like the CPU oracle's.
#define MC_REAL double
#include "mc_launch_impl.cuh"

#include "mc_matbuild.h"

namespace mcg {

// The temperature-dependent tables of n Materials that share dispersion
// and relaxation rows: block t builds temperature T[t]. Each bin's
// quantities come from the host/device formulas of mc_matbuild.h; the sums
// and running sums that depend on the order of their terms are taken in the
// host build's order by one thread each, so every output equals
// mc_material_create's bit for bit (this unit is compiled without
// contraction, --fmad=false).
__global__ void __launch_bounds__(256) k_build_materials(MatBuildArgs A) {
    const int t = blockIdx.x;
    const double T = A.T[t];
    const long nw = A.nw, np = A.np, nt = nw * np;
    double* tau = A.tau + (size_t)t * nt;
    double* epdf = A.scratch + (size_t)t * 3 * nt;
    double* fpdf = epdf + nt;
    double* spdf = fpdf + nt;
    double* rowF = A.rows + (size_t)t * 2 * nw;
    double* rowS = rowF + nw;
    unsigned long long* fwthr = A.fwthr + (size_t)t * nw;
    unsigned long long* swthr = A.swthr + (size_t)t * nw;
    unsigned long long* fpthr = A.fpthr + (size_t)t * nt;
    unsigned long long* spthr = A.spthr + (size_t)t * nt;
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (long w = threadIdx.x; w < nw; w += blockDim.x) {
        const double om = A.omega[w];
        const double dedT = dEdT(om, T);
        for (long p = 0; p < np; ++p) {
            const long i = w * np + p;
            const double ta = 1. / tauInverse(A.relax, p, om, T);
            tau[i] = ta;
            if (!isfinite(ta) || !(A.vel[i] > MAT_DMIN)) atomicOr(&bad, 1);
            const double e = dedT * A.dos[i] * A.domega[w];
            epdf[i] = e;
            fpdf[i] = A.vel[i] * e;
            spdf[i] = e / ta;
        }
        rowF[w] = branchThresholds(fpdf, w, np, fpthr);
        rowS[w] = branchThresholds(spdf, w, np, spthr);
    }
    __syncthreads();
    // order-dependent sums, one sequence per thread
    double* sums = A.sums + (size_t)t * 4;
    if (threadIdx.x < 4) {
        double s = 0.;
        for (long i = 0; i < nt; ++i) {
            const double e = epdf[i];
            s += threadIdx.x == 0 ? e
               : threadIdx.x == 1 ? A.vel[i] * e
               : threadIdx.x == 2 ? e / tau[i]
                                  : tau[i] * (A.vel[i] * A.vel[i]) * e;
        }
        sums[threadIdx.x] = threadIdx.x == 3 ? s / 3. : s;
    } else if (threadIdx.x == 32 || threadIdx.x == 64) {
        // running sums over the bins -> bin thresholds
        const double* row = threadIdx.x == 32 ? rowF : rowS;
        unsigned long long* thr = threadIdx.x == 32 ? fwthr : swthr;
        double acc = 0.;
        for (long w = 0; w < nw; ++w) acc += row[w];
        double pre = 0.;
        for (long w = 0; w < nw; ++w) {
            pre += row[w];
            thr[w] = cdfThreshold(pre / acc);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) A.status[t] = bad;
}

cudaError_t launchBuildMaterials(const MatBuildArgs& a, int n, cudaStream_t s) {
    k_build_materials<<<n, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mcg
