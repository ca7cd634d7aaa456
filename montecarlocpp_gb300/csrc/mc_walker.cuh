// mc_walker.cuh -- the phonon event loop shared by the single-instance and
// batched kernels: shared-memory layout, field tallies, the cell walk of a
// flight, emission, and Walker (one phonon in flight).
#pragma once

#include "mc_device.cuh"

namespace mcg {

// Shared fixed-point fields are cell-major with an odd stride of 64-bit
// words per cell (rows rounded up to odd), so the rows of a cell sit at
// fixed offsets and lanes that add to different cells spread over the
// banks; the difference array that follows has cols + 1 such cells.
__host__ __device__ inline int talStride(int rows) { return rows | 1; }
__host__ __device__ inline size_t talEntries(int rows, int cols) {
    return (size_t)talStride(rows) * (2 * (size_t)cols + 1);
}

// ---------------------------------------------------------------- tables
// Shared layout of a single-instance launch: vel and vel*tau tables, the
// scatter bin thresholds and guide table, the subdomains (when staged), the
// instance descriptor, then the block's tally.
struct SmemLayout {
    size_t vel = 0, vt = 0, wthr = 0, guide = 0, sd = 0, inst = 0, tal = 0, split = 0, total = 0;
    template <typename R>
    __host__ __device__ void init(int nw, int np, int nsdShared, int rows, int cols, bool sharedTally,
                                  bool splitTally = false, bool tabShared = true) {
        auto al = [](size_t b) { return (b + 15) & ~(size_t)15; };
        const size_t nt = (size_t)nw * np;
        vel = 0;
        vt = al(vel + sizeof(R) * nt);
        wthr = al(vt + (tabShared ? sizeof(R) * nt : 0));
        guide = al(wthr + sizeof(unsigned long long) * (size_t)nw);
        sd = al(guide + (tabShared ? sizeof(uint16_t) * GUIDE : 0));
        inst = al(sd + sizeof(SdomD<R>) * (size_t)nsdShared);
        tal = al(inst + sizeof(InstD<R>));
        total = tal + (sharedTally ? sizeof(long long) * talEntries(rows, cols) : 0);
        if (splitTally) {
            split = al(total);
            total = split + 2 * sizeof(unsigned) * talEntries(rows, cols);
        }
    }
};

// Shared layout of a single-instance advance launch (tables, every
// subdomain image, descriptor, fixed-point field when the tally is shared);
// the host sizes the launch with the same function.
// splitTally: the lean flights' carry-free field (below) after the tally.
template <typename R>
__host__ __device__ inline SmemLayout singleLayout(int nw, int np, int nsd, int rows, int cols, bool sharedTally,
                                                   bool splitTally = false, bool tabShared = true) {
    SmemLayout L;
    L.init<R>(nw, np, nsd, rows, cols, sharedTally, splitTally, tabShared);
    return L;
}

// Subdomain images a batched block stages in shared memory up to this many
// bytes.
constexpr size_t SD_SHARED_MAX = 32 * 1024;

// Shared memory of a batched block: the current instance's descriptor and
// tables, and room for the largest subdomain images and fixed-point field
// that any instance of the launch stages.
struct BatchSmem {
    size_t inst = 0, vel = 0, vt = 0, wthr = 0, guide = 0, sd = 0, tal = 0, total = 0;
    template <typename R>
    __host__ __device__ void init(int nt, int nw, int sdBytes, int talEntries) {
        auto al = [](size_t b) { return (b + 15) & ~(size_t)15; };
        inst = 0;
        vel = al(sizeof(InstD<R>));
        vt = al(vel + sizeof(R) * (size_t)nt);
        wthr = al(vt + sizeof(R) * (size_t)nt);
        guide = al(wthr + sizeof(unsigned long long) * (size_t)nw);
        sd = al(guide + sizeof(uint16_t) * GUIDE);
        tal = al(sd + (size_t)sdBytes);
        total = tal + sizeof(long long) * (size_t)talEntries;
    }
};

// Fixed-point fields a batched block keeps in shared memory up to this size
// (larger ones go straight to the global field).
constexpr size_t TAL_BATCH_MAX = 32 * 1024;
// Shared memory a batched FP32 block may use with subdomains staged (four
// resident blocks per SM); FP64 blocks (two per SM) may use twice this.
constexpr size_t BATCH_SMEM_F32 = 56 * 1024;

__host__ __device__ inline size_t smemTallyBytes(int rows, int cols) {
    return sizeof(long long) * talEntries(rows, cols);
}

// Tally modes: per-block shared histogram (64-bit fixed point, exact and
// order-independent adds) flushed with FP64 atomics, or FP64 atomics
// straight to the global field (fields too large for shared memory), or
// either per instance (batched launches: shared when InstD::tal is set).
enum { TM_SHARED = 0, TM_GLOBAL = 1, TM_AUTO = 2, TM_NONE = 3 };
// (TM_NONE: batched launches whose instances keep no field, only the
// per-flight checksums -- the flight code without any field path.)

// Hard cap on events one thread processes in one launch (a guard: a
// phonon that reaches it is killed and flagged non-finite).
constexpr int MAX_EVENTS_PER_LAUNCH = 1 << 22;

// Resident blocks of 256 threads per SM the FP32 advance kernels are
// compiled for (register budget 65536 / (256 x this)): three (80
// registers) measured faster than four (64, with spills) on the fused
// kernels.
#ifndef MC_MIN_BLOCKS_F32
#define MC_MIN_BLOCKS_F32 3
#endif
// Resident blocks of the FP32 static kernel per SM: one block of 768
// consumer threads and a producer warp. Three blocks of 256 consumers (the
// same warps per SM) measured 4 % slower over a whole horizon: each block
// streams its own region, and an SM whose first block finished early ran
// its last block with a third of the warps (blocks' finishing times spread
// over 20 % of a launch); one block per SM shares its tiles among all the
// SM's warps, so they finish together.
#ifndef MC_MIN_BLOCKS_STATIC_F32
#define MC_MIN_BLOCKS_STATIC_F32 1
#endif
// The static kernel's consumer threads per block at most (and its default
// block size) in FP32 and in FP64 flight (two resident blocks of 256 leave
// the FP64 walker its registers), its shared-memory stages of the state
// stream, and whether it reads the vel * tau and guide tables (used at
// scatters only) from global memory instead of staging them, which leaves
// room for more stages.
#ifndef MC_STATIC_CONSUMERS
#define MC_STATIC_CONSUMERS 768
#endif
#ifndef MC_STATIC_CONSUMERS_F64
#define MC_STATIC_CONSUMERS_F64 256
#endif
#ifndef MC_STATIC_STAGES
#define MC_STATIC_STAGES 2
#endif
#ifndef MC_STATIC_TABLES_GLOBAL
#define MC_STATIC_TABLES_GLOBAL 0
#endif
// Programmatic dependent launch of the static kernel: launch k + 1's blocks
// stage their tables and initialise their barriers while launch k's last
// blocks finish, and wait for launch k to complete before they touch the
// state, the region counts or the field.
#ifndef MC_PDL
#define MC_PDL 1
#endif
// Single-instance dynamic launches of long windows claim slots from one
// launch-wide counter (else each block from its own share).
#ifndef MC_DYN_GLOBAL_QUEUE
#define MC_DYN_GLOBAL_QUEUE 1
#endif
// dt-steps per window from which a launch uses that counter
#ifndef MC_DYN_QUEUE_MIN_STEPS
#define MC_DYN_QUEUE_MIN_STEPS 1024
#endif
// Constant tables staged by bulk copies (else by the threads, one element
// per thread per loop iteration).
#ifndef MC_TABLE_BULK
#define MC_TABLE_BULK 1
#endif

template <typename R>
struct Phn {
    int s;          // subdomain
    int idx[3];     // cell
    R off[3];       // offset inside the cell, in [0, 1]
    R d[3];         // direction (unit, physical)
    R scatNext;
    int w, p;
    bool neg;       // sign -1
    uint32_t nscat, nloop, id;
};

// Fixed-point amount of a flight. FP32 flight: the quantum gives the
// largest single flight 2^27 units, so one 32-bit round-to-nearest
// conversion suffices (|v| < 2^31); sums are kept in 64 bits. FP64 flight:
// 64-bit conversion against a quantum sized for a block's total.
__device__ __forceinline__ int toFixed(float v) { return __float2int_rn(v); }
__device__ __forceinline__ long long toFixed(double v) { return __double2ll_rn(v); }
// fixed-point amount of one flight in each flight precision
template <typename R> struct FixT;
template <> struct FixT<float> { using T = int; };
template <> struct FixT<double> { using T = long long; };

// float -> double by moving the bits (the conversion instruction runs on
// GB300's narrow FP64 pipe); zero and subnormal inputs give zero.
__device__ __forceinline__ double toDouble(float v) {
    const uint32_t b = __float_as_uint(v);
    const uint32_t e = (b >> 23) & 0xFFu;
    if (e == 0u) return 0.0;
    const uint32_t m = b & 0x7FFFFFu;
    const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | (m >> 3);
    return __hiloint2double((int)hi, (int)(m << 29));
}
__device__ __forceinline__ double toDouble(double v) { return v; }

// Exact 64-bit add into a word of shared memory with native 32-bit atomics
// (a 64-bit add on a shared address compiles to a compare-and-swap loop):
// the low half takes the low 32 bits of v, and the high half the sign
// extension of v plus the carry out of the low half, skipped when they
// cancel (always, for the |v| < 2^31 of an FP32 flight, unless the low half
// wraps). The two halves are consistent again once every add has landed,
// which the callers' barriers ensure before any read.
__device__ __forceinline__ void sharedAdd64(long long* p, long long v) {
    unsigned* w = reinterpret_cast<unsigned*>(p);
    const unsigned lo = (unsigned)(unsigned long long)v;
    const unsigned old = atomicAdd(w, lo);
    const int hi = (int)(v >> 32) + ((old + lo) < old ? 1 : 0);
    if (hi != 0) atomicAdd(reinterpret_cast<int*>(w + 1), hi);
}
// the same for a 32-bit amount (sign extension from bit 31)
__device__ __forceinline__ void sharedAdd64(long long* p, int v) {
    unsigned* w = reinterpret_cast<unsigned*>(p);
    const unsigned lo = (unsigned)v;
    const unsigned old = atomicAdd(w, lo);
    const int hi = (v >> 31) + ((old + lo) < old ? 1 : 0);
    atomicAdd(reinterpret_cast<int*>(w + 1), hi);  // unconditional: no branch
}
__device__ __forceinline__ void sharedAdd64(unsigned long long* p, unsigned long long v) {
    sharedAdd64(reinterpret_cast<long long*>(p), (long long)v);
}

// Per-block accumulators in shared memory: the launch counters and the
// rows' fixed-point checksums of the flights whose field amount does not go
// into the block's shared field (those are summed from it at the end).
struct BlockAcc {
    unsigned long long cnt[C_NCOUNTERS];
    long long csum[4];
};
static __shared__ BlockAcc g_blk;

// Add n to block counter c, summed first over the lanes of the warp that
// reach this point together with the same c (one shared atomic per group).
__device__ __forceinline__ void blkCount(int c, unsigned n) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, c);
    const unsigned tot = __reduce_add_sync(peers, n);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && tot) sharedAdd64(&g_blk.cnt[c], (unsigned long long)tot);
}

// Add v to the block checksum of row r, summed first over the lanes that
// reach this point together (all with the same r): three 22-bit limbs keep
// the 32-bit warp sums exact.
__device__ __forceinline__ void blkCsum(int r, long long v) {
    const unsigned act = __activemask();
    const unsigned long long u = (unsigned long long)v;
    const int s0 = __reduce_add_sync(act, (int)(u & 0x3FFFFFull));
    const int s1 = __reduce_add_sync(act, (int)((u >> 22) & 0x3FFFFFull));
    const int s2 = __reduce_add_sync(act, (int)(v >> 44));
    if ((int)(threadIdx.x & 31) == __ffs(act) - 1) {
        const long long t = (long long)s0 + (long long)s1 * (1LL << 22) + (long long)s2 * (1LL << 44);
        if (t != 0) sharedAdd64(&g_blk.csum[r], t);
    }
}

// Zero the block accumulators (all threads; a barrier must follow).
__device__ __forceinline__ void blkZero() {
    unsigned long long* z = reinterpret_cast<unsigned long long*>(&g_blk);
    for (int i = threadIdx.x; i < (int)(sizeof(BlockAcc) / 8); i += blockDim.x) z[i] = 0ull;
}

// Instance data of the advance loop, read through a view. A batched launch
// reads the descriptor of the phonon's instance that its block staged in
// shared memory (InstView). A single-instance launch (ParamView) takes the
// launch constants from the kernel parameters and its tables, subdomain
// images and fixed-point field from its own shared-memory layout, at
// addresses the compiler knows to be shared: no pointer is loaded from
// memory on the way, so nothing has to be reloaded after a tally atomic.
template <typename R>
struct InstView {
    const InstD<R>* I;
    __device__ __forceinline__ int rows() const { return I->rows; }
    __device__ __forceinline__ int cols() const { return I->cols; }
    __device__ __forceinline__ int problem() const { return I->problem; }
    __device__ __forceinline__ int cumStep() const { return I->cumStep; }
    __device__ __forceinline__ int nw() const { return I->nw; }
    __device__ __forceinline__ int np() const { return I->np; }
    __device__ __forceinline__ bool talShared() const { return I->tal != nullptr; }
    __device__ __forceinline__ long long* tal() const { return I->tal; }
    __device__ __forceinline__ long long* dif() const { return I->dif; }
    __device__ __forceinline__ double* tally() const { return I->tally; }
    __device__ __forceinline__ double* gdif() const { return I->gdif; }
    __device__ __forceinline__ int groups() const { return I->groups; }
    __device__ __forceinline__ long long gstride() const { return I->gstride; }
    __device__ __forceinline__ int flags() const { return I->flags; }
    __device__ __forceinline__ R tqinv(int r) const { return I->tqinv[r]; }
    __device__ __forceinline__ const SdomD<R>* sd() const { return I->sd; }
    __device__ __forceinline__ const R* vel() const { return I->vel; }
    __device__ __forceinline__ const R* vt() const { return I->vt; }
    __device__ __forceinline__ const unsigned long long* wthr() const { return I->wthr; }
    __device__ __forceinline__ const uint16_t* wguide() const { return I->wguide; }
    __device__ __forceinline__ const unsigned long long* pthr() const { return I->pthr; }
    __device__ __forceinline__ uint32_t key0() const { return I->key0; }
    __device__ __forceinline__ uint32_t key1() const { return I->key1; }
    __device__ __forceinline__ long long maxscat() const { return I->maxscat; }
    __device__ __forceinline__ long long maxloop() const { return I->maxloop; }
};

// Single-instance view over singleLayout(), whose offsets the host puts in
// the launch parameters (setSingleLayout).
template <typename R, int TM>
struct ParamView {
    const Params<R>* P;
    unsigned char* sm;
    __device__ __forceinline__ void init(const Params<R>& p, unsigned char* smraw) {
        P = &p;
        sm = smraw;
    }
    __device__ __forceinline__ int rows() const { return P->rows; }
    __device__ __forceinline__ int cols() const { return P->cols; }
    __device__ __forceinline__ int problem() const { return P->problem; }
    __device__ __forceinline__ int cumStep() const { return P->cumStep; }
    __device__ __forceinline__ int nw() const { return P->nw; }
    __device__ __forceinline__ int np() const { return P->np; }
    __device__ __forceinline__ bool talShared() const { return TM == TM_SHARED; }
    __device__ __forceinline__ long long* tal() const {
        return TM == TM_SHARED ? reinterpret_cast<long long*>(sm + P->smTal) : nullptr;
    }
    __device__ __forceinline__ long long* dif() const {
        return reinterpret_cast<long long*>(sm + P->smTal) + (size_t)talStride(P->rows) * P->cols;
    }
    // the carry-free field of the lean flights: low 16-bit parts, then the
    // high parts, one 32-bit word each per entry of the 64-bit field
    __device__ __forceinline__ unsigned* split() const { return reinterpret_cast<unsigned*>(sm + P->smSplit); }
    __device__ __forceinline__ int entries() const { return (int)talEntries(P->rows, P->cols); }
    __device__ __forceinline__ double* tally() const { return P->tally; }
    __device__ __forceinline__ double* gdif() const { return nullptr; }
    __device__ __forceinline__ int groups() const { return 1; }
    __device__ __forceinline__ long long gstride() const { return 0; }
    __device__ __forceinline__ int flags() const { return 0; }
    __device__ __forceinline__ R tqinv(int r) const { return P->tqinv[r]; }
    __device__ __forceinline__ const SdomD<R>* sd() const { return reinterpret_cast<const SdomD<R>*>(sm + P->smSd); }
    __device__ __forceinline__ const R* vel() const { return reinterpret_cast<const R*>(sm); }
    __device__ __forceinline__ const R* vt() const {
        return P->tabGlobal ? P->vt : reinterpret_cast<const R*>(sm + P->smVt);
    }
    __device__ __forceinline__ const unsigned long long* wthr() const {
        return reinterpret_cast<const unsigned long long*>(sm + P->smWthr);
    }
    __device__ __forceinline__ const uint16_t* wguide() const {
        return P->tabGlobal ? P->wguide : reinterpret_cast<const uint16_t*>(sm + P->smGuide);
    }
    __device__ __forceinline__ const unsigned long long* pthr() const { return P->pthr; }
    __device__ __forceinline__ uint32_t key0() const { return P->key0; }
    __device__ __forceinline__ uint32_t key1() const { return P->key1; }
    __device__ __forceinline__ long long maxscat() const { return P->maxscat; }
    __device__ __forceinline__ long long maxloop() const { return P->maxloop; }
};

// Batched view: the instance a block is bound to, as it staged it. The
// descriptor's scalars come from the staged copy; the tables (always
// staged) and the fixed-point field (when the instance stages one) sit at
// the batched layout's offsets, which the host puts in the launch
// parameters (setBatchLayout), so they are shared-memory accesses with
// known addresses; the subdomain images stay behind the descriptor's
// pointer (shared or global, per instance).
template <typename R>
struct BatchView {
    const Params<R>* P;
    unsigned char* sm;
    const InstD<R>* I;
    __device__ __forceinline__ int rows() const { return I->rows; }
    __device__ __forceinline__ int cols() const { return I->cols; }
    __device__ __forceinline__ int problem() const { return I->problem; }
    __device__ __forceinline__ int cumStep() const { return I->cumStep; }
    __device__ __forceinline__ int nw() const { return I->nw; }
    __device__ __forceinline__ int np() const { return I->np; }
    __device__ __forceinline__ bool talShared() const { return (I->flags & IF_TAL_SHARED) != 0; }
    __device__ __forceinline__ long long* tal() const { return reinterpret_cast<long long*>(sm + P->smTal); }
    __device__ __forceinline__ long long* dif() const {
        return reinterpret_cast<long long*>(sm + P->smTal) + (size_t)talStride(I->rows) * I->cols;
    }
    __device__ __forceinline__ double* tally() const { return I->tally; }
    __device__ __forceinline__ double* gdif() const { return I->gdif; }
    __device__ __forceinline__ int groups() const { return I->groups; }
    __device__ __forceinline__ long long gstride() const { return I->gstride; }
    __device__ __forceinline__ int flags() const { return I->flags; }
    __device__ __forceinline__ R tqinv(int r) const { return I->tqinv[r]; }
    __device__ __forceinline__ const SdomD<R>* sd() const { return I->sd; }
    __device__ __forceinline__ const R* vel() const { return reinterpret_cast<const R*>(sm + P->smVel); }
    __device__ __forceinline__ const R* vt() const { return reinterpret_cast<const R*>(sm + P->smVt); }
    __device__ __forceinline__ const unsigned long long* wthr() const {
        return reinterpret_cast<const unsigned long long*>(sm + P->smWthr);
    }
    __device__ __forceinline__ const uint16_t* wguide() const { return reinterpret_cast<const uint16_t*>(sm + P->smGuide); }
    __device__ __forceinline__ const unsigned long long* pthr() const { return I->pthr; }
    __device__ __forceinline__ uint32_t key0() const { return I->key0; }
    __device__ __forceinline__ uint32_t key1() const { return I->key1; }
    __device__ __forceinline__ long long maxscat() const { return I->maxscat; }
    __device__ __forceinline__ long long maxloop() const { return I->maxloop; }
};

// Field accumulation for one flight of one instance.
// SPLIT (FP32 lean flights only): adds go to a carry-free copy of the
// shared field instead -- the low 14 bits of the amount into one 32-bit
// word, the rest (arithmetic shift) into another, both without a returned
// value. A lean flight adds to an entry at most once, |amount| < 2^27, and
// a block runs at most regCap <= 2^18 of them per launch, so neither word
// can overflow (2^18 x (2^14 - 1) < 2^32 unsigned; 2^18 x 2^13 = 2^31
// signed, reached only by the most negative amounts); closeBlock folds the
// copy into the 64-bit field.
constexpr int SPLIT_LOW_BITS = 14;
constexpr unsigned SPLIT_LOW_MASK = (1u << SPLIT_LOW_BITS) - 1u;
// lean flights per block per launch the carry-free copy holds exactly
constexpr long long SPLIT_MAX_FLIGHTS = 262144;

template <typename R, int TM, typename IA, bool SPLIT = false>
struct Tally {
    IA V;
    long long goff;  // offset of the phonon's field copy (global layouts)
    // amount per metre of flight of the flight's nAct rows, which are field
    // rows rowBase .. rowBase + nAct - 1: Temp sign/v; Flux sign*d; Multi
    // both; CumTemp / CumFlux those of the flight's scatter-count bin
    R rho[4];
    int nAct, rowBase;

    __device__ __forceinline__ int rows() const { return V.rows(); }
    __device__ __forceinline__ bool shared() const {
        return TM == TM_SHARED || (TM == TM_AUTO && V.talShared());
    }
    using Fix = typename FixT<R>::T;
    // fixed-point amount of row r for path length t
    __device__ __forceinline__ Fix fixedOf(int r, R t) const { return toFixed(rho[r] * (t * V.tqinv(r))); }
    // a flight's amount that does not enter the shared field
    __device__ __forceinline__ void csumAdd(int r, long long v) const { blkCsum(r, v); }
    // shared field and difference array, cell-major: row r of column c at
    // [c * talStride(rows) + r]
    __device__ __forceinline__ void splitAdd(int e, Fix v) const {
        unsigned* lo = V.split();
        atomicAdd(lo + e, (unsigned)v & SPLIT_LOW_MASK);
        atomicAdd(reinterpret_cast<int*>(lo) + V.entries() + e, (int)(v >> SPLIT_LOW_BITS));
    }
    __device__ __forceinline__ void atomShared(int r, int col, Fix v) const {
        if constexpr (SPLIT) splitAdd(col * talStride(V.rows()) + rowBase + r, v);
        else sharedAdd64(&V.tal()[col * talStride(V.rows()) + rowBase + r], v);
    }
    __device__ __forceinline__ void atomRange(int r, int c0, int c1, Fix v) const {
        const int st = talStride(V.rows());
        if constexpr (SPLIT) {
            const int d = st * V.cols() + rowBase + r;
            splitAdd(d + c0 * st, v);
            splitAdd(d + c1 * st, -v);
        } else {
            long long* d = V.dif() + rowBase + r;
            sharedAdd64(d + c0 * st, v);
            sharedAdd64(d + c1 * st, -v);
        }
    }
    __device__ __forceinline__ void addGlobal(int col, R t) const {
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < nAct)
                atomicAdd(&V.tally()[goff + (size_t)col * V.rows() + rowBase + r], toDouble(rho[r] * t));
    }
    // interior cells [c0, c1) of a 1-D walk (stride 1) each with path t
    __device__ __forceinline__ void addGlobalRange(int c0, int c1, R t) const {
        if (V.gdif()) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (r < nAct) {
                    const double v = toDouble(rho[r] * t);
                    const size_t row = (size_t)(rowBase + r) * (V.cols() + 1);
                    atomicAdd(&V.gdif()[goff + row + c0], v);
                    atomicAdd(&V.gdif()[goff + row + c1], -v);
                }
            }
        } else {
            for (int c = c0; c < c1; ++c) addGlobal(c, t);
        }
    }
};

// The rows a flight adds to (montecarlo/problem.cpp:473-544,589-633, each
// amount times the phonon's sign): the per-metre amounts rho and the rows'
// place in the field, from the phonon's sign, 1/v, direction and scatter
// count before the flight.
template <typename R, int TM, typename IA, bool SPLIT>
__device__ __forceinline__ void setFlightRows(Tally<R, TM, IA, SPLIT>& T, int problem, bool neg, R iv, const R d[3],
                                              uint32_t nscat, int cumStep) {
    const R sg = neg ? R(-1) : R(1);
    T.rowBase = 0;
    if (problem == P_TEMP) { T.nAct = 1; T.rho[0] = sg * iv; T.rho[1] = T.rho[2] = T.rho[3] = R(0); }
    else if (problem == P_FLUX) { T.nAct = 3; T.rho[0] = sg * d[0]; T.rho[1] = sg * d[1]; T.rho[2] = sg * d[2]; T.rho[3] = R(0); }
    else if (problem == P_MULTI) { T.nAct = 4; T.rho[0] = sg * iv; T.rho[1] = sg * d[0]; T.rho[2] = sg * d[1]; T.rho[3] = sg * d[2]; }
    else {
        // nscat < maxscat < 2^31 and cumStep < 2^31 (checked on the host)
        const int bin = (int)((nscat + (uint32_t)cumStep - 1u) / (uint32_t)cumStep);
        if (problem == P_CUMTEMP) {
            T.nAct = 1; T.rowBase = bin;
            T.rho[0] = sg * iv; T.rho[1] = T.rho[2] = T.rho[3] = R(0);
        } else {
            T.nAct = 3; T.rowBase = 3 * bin;
            T.rho[0] = sg * d[0]; T.rho[1] = sg * d[1]; T.rho[2] = sg * d[2]; T.rho[3] = R(0);
        }
    }
}

// Reduced velocity a = S (M^-1 d) and its reciprocal.
template <typename R>
__device__ __forceinline__ void reducedVel(const SdomD<R>& S, const R d[3], R a[3], R ia[3]) {
    R m[3];
    rotate(S.Minv, d, m);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = S.S[k] * m[k];
        ia[k] = R(1) / a[k];
    }
}

template <typename R>
__device__ __forceinline__ R clamp01(R x) { return fmin(fmax(x, R(0)), R(1)); }

// Move along axis k by du cells (no tally): displacement relative to the
// current cell, then re-split into cell index and offset.
template <typename R>
__device__ __forceinline__ void moveAxis(Phn<R>& ph, const SdomD<R>& S, int k, R du) {
    const int sh = (int)floor(du);
    const int i = min(max(ph.idx[k] + sh, 0), S.shape[k] - 1);
    ph.off[k] = clamp01(du - (R)(i - ph.idx[k]));
    ph.idx[k] = i;
}

// Component k of a 3-vector by selects (no indexed access, so the vector
// stays in registers whatever k is).
template <typename T>
__device__ __forceinline__ T pick3(const T v[3], int k) {
    return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]);
}

// 1-D flight along axis K (the only axis with cells): closed form of
// montecarlo/field.cpp:187-223 -- partial first and last cells, full
// interior cells through the difference array. In the shared layout the
// flight's whole fixed-point amount V is computed once and the last cell
// takes the integer remainder, so the cells add up to V exactly. Called
// with a constant K the selects fold away (one copy per axis); with a
// run-time K one copy serves every axis.
template <typename R, int TM, typename IA, bool SPLIT = false>
__device__ __forceinline__ void fly1d(Phn<R>& ph, const SdomD<R>& S, const R a[3], const R ia[3], R s,
                                      Tally<R, TM, IA, SPLIT>& T, const int K) {
    const int cb = S.colbeg;
    const int b = pick3(ph.idx, K);
    const int n = S.shape[K];
    const R offK = pick3(ph.off, K);
    // displacement in cell units relative to the current cell
    const R du = offK + s * pick3(a, K);
    int e = b + (int)floor(du);
    e = min(max(e, 0), n - 1);
    const int stride = S.tstride[K];
    const R inva = fabs(pick3(ia, K));
    const int lo = min(b, e), hi = max(b, e);
    const int nin = hi - lo - 1;  // interior cells; -1 when the flight stays in its cell
    const R tfirst = (e > b ? (R(1) - offK) : offK) * inva;
    using Fix = typename FixT<R>::T;
    if (T.shared()) {
        // the first cell's add is common to every lane (all of V when the
        // flight stays in its cell), the others only add to it: no lane
        // waits for another's branch
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (r < T.nAct) {
                const Fix V = T.fixedOf(r, s);
                const Fix F = T.fixedOf(r, tfirst);
                const Fix I = T.fixedOf(r, inva);
                T.atomShared(r, cb + b * stride, e == b ? V : F);
                if (e != b) T.atomShared(r, cb + e * stride, V - F - (Fix)nin * I);
                if (nin > 0) {
                    if (stride == 1) {
                        T.atomRange(r, cb + lo + 1, cb + hi, I);
                    } else {
                        for (int c = lo + 1; c < hi; ++c) T.atomShared(r, cb + c * stride, I);
                    }
                }
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < T.nAct) T.csumAdd(r, T.fixedOf(r, s));
    }
    if (!T.shared()) {
        if (e == b) {
            T.addGlobal(cb + b * stride, s);
        } else {
            const R tlast = s - tfirst - (R)(hi - lo - 1) * inva;
            T.addGlobal(cb + b * stride, tfirst);
            T.addGlobal(cb + e * stride, fmax(tlast, R(0)));
            if (stride == 1) { if (hi - lo > 1) T.addGlobalRange(cb + lo + 1, cb + hi, inva); }
            else for (int c = lo + 1; c < hi; ++c) T.addGlobal(cb + c * stride, inva);
        }
    }
    const R offNew = clamp01(du - (R)(e - b));
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (j == K) { ph.idx[j] = e; ph.off[j] = offNew; }
        else moveAxis(ph, S, j, ph.off[j] + s * a[j]);
    }
}

// Flight of path length s from the current cell, tallied cell by cell
// (Field::accumulate, montecarlo/field.cpp:160-288, as a cell walk); adds
// the flight's fixed-point amount to the checksums.
// COMPACT: one run-time-axis copy of the 1-D flight instead of one per
// axis (smaller code for kernels that run the walker rarely).
template <typename R, int TM, typename IA, bool COMPACT>
__device__ __forceinline__ void fly(Phn<R>& ph, const SdomD<R>& S, const R a[3], const R ia[3], R s,
                                   Tally<R, TM, IA>& T) {
    const int acc = (TM == TM_NONE || (TM == TM_AUTO && (T.V.flags() & IF_NO_FIELD))) ? -2 : S.accum;
    const int cb = S.colbeg;
    if (acc < 0) {
        // a single field column (or none): move only
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (r < T.nAct) {
                const typename FixT<R>::T V = T.fixedOf(r, s);
                if (acc == -1 && T.shared()) T.atomShared(r, cb, V);
                else T.csumAdd(r, V);
            }
        }
        if (acc == -1 && !T.shared()) T.addGlobal(cb, s);
#pragma unroll
        for (int k = 0; k < 3; ++k) moveAxis(ph, S, k, ph.off[k] + s * a[k]);
        return;
    }
    if (COMPACT) {
        if (acc <= 2) { fly1d<R, TM, IA>(ph, S, a, ia, s, T, acc); return; }
    } else {
        if (acc == 0) { fly1d<R, TM, IA>(ph, S, a, ia, s, T, 0); return; }
        if (acc == 1) { fly1d<R, TM, IA>(ph, S, a, ia, s, T, 1); return; }
        if (acc == 2) { fly1d<R, TM, IA>(ph, S, a, ia, s, T, 2); return; }
    }
    // 2-D / 3-D: walk the cells (Amanatides-Woo); a shared field gives the
    // checksum as the sum of its cells, a global one the flight's amount
    if (!T.shared()) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < T.nAct) T.csumAdd(r, T.fixedOf(r, s));
    }
    R rem = s;
    // the lanes that walk: each leaves the loop after its own number of
    // crossings; they wait for one another after it, so that the event code
    // that follows runs once for all of them rather than once per exit
    // (measured: 4.2 of 32 lanes active per instruction on the pore cell
    // without it, the kernel 2.1x slower; a walk that shares all lanes'
    // segments out over the warp gained a further 2% only, for spilled
    // registers)
    const unsigned walkers = __activemask();
    const int s0 = S.tstride[1], s01 = S.tstride[2];
    for (int guard = 0; guard < 3 * MAX_SHAPE + 4; ++guard) {
        R tmin = rem;
        int ax = -1;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R t = tmin;
            if (a[k] > R(0) && ph.idx[k] < S.shape[k] - 1) t = (R(1) - ph.off[k]) * ia[k];
            else if (a[k] < R(0) && ph.idx[k] > 0) t = -ph.off[k] * ia[k];
            if (t < tmin) { tmin = t; ax = k; }
        }
        tmin = fmax(tmin, R(0));
        const int col = cb + ph.idx[0] * S.tstride[0] + ph.idx[1] * s0 + ph.idx[2] * s01;
        if (T.shared()) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (r < T.nAct) T.atomShared(r, col, T.fixedOf(r, tmin));
        } else {
            T.addGlobal(col, tmin);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ph.off[k] = clamp01(ph.off[k] + tmin * a[k]);
            if (k == ax) {
                if (a[k] > R(0)) { ph.idx[k] += 1; ph.off[k] = R(0); }
                else { ph.idx[k] -= 1; ph.off[k] = R(1); }
            }
        }
        rem -= tmin;
        if (ax < 0) break;
    }
    __syncwarp(walkers);
}

template <typename R>
__device__ __forceinline__ void physPos(const SdomD<R>& S, const Phn<R>& ph, double x[3]) {
    double u[3];
    for (int k = 0; k < 3; ++k) u[k] = ((double)ph.idx[k] + (double)ph.off[k]) / (double)S.S[k];
    for (int r = 0; r < 3; ++r)
        x[r] = (double)S.o[r] + (((double)S.M[3 * r] * u[0] + (double)S.M[3 * r + 1] * u[1]) +
                                 (double)S.M[3 * r + 2] * u[2]);
}

template <typename R>
__device__ __forceinline__ void logEvent(const Params<R>& P, const Phn<R>& ph, int sBefore, int face,
                                         int sAfter, double xEnd[3], double time, int cellEnd) {
    if (P.log == nullptr || (long long)ph.id >= P.logn) return;
    long long i = ph.nloop;
    if (i >= P.logcap) return;
    double* r = P.log + ((long long)ph.id * P.logcap + i) * 12;
    r[0] = (double)ph.nloop; r[1] = sBefore; r[2] = face; r[3] = sAfter; r[4] = cellEnd;
    r[5] = xEnd[0]; r[6] = xEnd[1]; r[7] = xEnd[2]; r[8] = time; r[9] = (double)ph.nscat;
    r[10] = ph.w; r[11] = ph.p;
    atomicMax(&P.logcount[ph.id], (int)(i + 1));
}

// drawScatNext (montecarlo/material.cpp:287-296): d = v tau (-log(1 - u)),
// redrawn while below the smallest normal number.
template <typename R, typename G>
__device__ __forceinline__ R drawScatNext(G& g, R vt) {
    R dist = R(0);
    for (int guard = 0; guard < 64 && dist < Lim<R>::tiny(); ++guard) dist = vt * neglog1m(g.next(), R(0));
    return dist;
}

// FieldProblem::solve emission part (montecarlo/problem.cpp:386-399) and
// Emitter::emit (montecarlo/boundary.cpp:378-385) for phonon `n` of
// instance I (event 0 of its random stream).
template <typename R, typename G>
__device__ __forceinline__ void emitOne(const InstD<R>& I, long long n, G& g, Phn<R>& ph) {
    // emitter = upper_bound(emitCdf, n)
    int lo = 0, hi = I.nem;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (I.emitCdf[mid] <= n) lo = mid + 1; else hi = mid;
    }
    const EmitterD& E = I.em[lo];
    const SdomD<R>& S = I.sd[E.sdom];
    g.setEvent(0);
    ph.s = E.sdom;
    ph.id = (uint32_t)n;
    ph.nscat = 0; ph.nloop = 0;
    {   // drawFluxProp (montecarlo/material.cpp:277-280)
        uint32_t x1 = g.next(), x2 = g.next();
        ph.w = searchThr(I.fwthr, I.nw, x1);
        ph.p = searchBranch(I.fpthr + (size_t)ph.w * I.np, I.np, x2);
    }
    R u[3];
    R dir[3];
    if (E.fold >= 0) {
        // a shape other than the Parallelepiped: the piece (Polygon
        // triangle, Prism / Pyramid sub-volume), then the folded uniforms
        // (montecarlo/subdomain.cpp:309-373,399-441,
        // montecarlo/boundary.cpp:180-186,246-256)
        int k = 0;
        if (E.npiece > 1) {
            const unsigned long long x = g.next();
            while (k < E.npiece - 1 && x >= E.thr[k]) ++k;
        }
        R c0 = u01<R>(g.next()), c1 = u01<R>(g.next());
        R c2 = E.ncoord == 3 ? u01<R>(g.next()) : R(0);
        if (E.fold == FOLD_TRIANGLE) {
            if (!(c0 + c1 < R(1))) { c0 = R(1) - c0; c1 = R(1) - c1; }
        } else if (E.fold == FOLD_PRISM || E.fold == FOLD_TETRA) {
            if (c0 + c1 > R(1)) { c0 = R(1) - c0; c1 = R(1) - c1; }
            if (E.fold == FOLD_TETRA) {
                if (c1 + c2 > R(1)) {
                    const R t = c2;
                    c2 = R(1) - c0 - c1;
                    c1 = R(1) - t;
                } else if (c0 + c1 + c2 > R(1)) {
                    const R t = c2;
                    c2 = c0 + c1 + c2 - R(1);
                    c0 = R(1) - c1 - t;
                }
            }
        }
        const double cc[3] = {(double)c0, (double)c1, (double)c2};
#pragma unroll
        for (int r = 0; r < 3; ++r)
            u[r] = (R)(E.U0[k][r] + ((E.L[k][3 * r] * cc[0] + E.L[k][3 * r + 1] * cc[1]) + E.L[k][3 * r + 2] * cc[2]));
        R v[3];
        if (E.face >= 0) {
            const FaceD<R>& F = S.f[E.face];
            drawAniso<R>(g, false, v);
            rotate(F.rot, v, dir);
            ph.neg = !(F.T >= R(0));
        } else {
            drawAniso<R>(g, true, v);
            rotate(S.grot, v, dir);
            ph.neg = !(((dir[0] * S.gradT[0] + dir[1] * S.gradT[1]) + dir[2] * S.gradT[2]) < R(0));
        }
    } else if (E.face >= 0) {
        // EmitBoundary: position on the face (montecarlo/boundary.cpp:147-152,
        // 418-421), cosine direction about the inward normal (423-426)
        const FaceD<R>& F = S.f[E.face];
        R r1 = u01<R>(g.next()), r2 = u01<R>(g.next());
        // (i, j) shape axes of each face (montecarlo/subdomain.h:149-154)
        switch (E.face) {
        case 0: u[0] = R(0); u[1] = r1 * S.S[1]; u[2] = r2 * S.S[2]; break;
        case 1: u[1] = R(0); u[2] = r1 * S.S[2]; u[0] = r2 * S.S[0]; break;
        case 2: u[2] = R(0); u[0] = r1 * S.S[0]; u[1] = r2 * S.S[1]; break;
        case 3: u[0] = S.S[0]; u[2] = r1 * S.S[2]; u[1] = r2 * S.S[1]; break;
        case 4: u[1] = S.S[1]; u[0] = r1 * S.S[0]; u[2] = r2 * S.S[2]; break;
        default: u[2] = S.S[2]; u[1] = r1 * S.S[1]; u[0] = r2 * S.S[0]; break;
        }
        R v[3];
        drawAniso<R>(g, false, v);
        rotate(F.rot, v, dir);
        ph.neg = !(F.T >= R(0));
    } else {
        // EmitSubdomain (montecarlo/subdomain.cpp:250-263,275-281)
        R c0 = u01<R>(g.next()), c1 = u01<R>(g.next()), c2 = u01<R>(g.next());
        u[0] = c0 * S.S[0]; u[1] = c1 * S.S[1]; u[2] = c2 * S.S[2];
        R v[3];
        drawAniso<R>(g, true, v);
        rotate(S.grot, v, dir);
        ph.neg = !(((dir[0] * S.gradT[0] + dir[1] * S.gradT[1]) + dir[2] * S.gradT[2]) < R(0));
    }
    normalize(dir);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int i = (int)floor(u[k]);
        i = min(max(i, 0), S.shape[k] - 1);
        ph.idx[k] = i;
        ph.off[k] = u[k] - (R)i;
        ph.d[k] = dir[k];
    }
    ph.scatNext = drawScatNext<R>(g, I.vt[ph.w * I.np + ph.p]);
}

template <typename R>
__device__ __forceinline__ void packPhonon(const Phn<R>& ph, typename Vec4<R>::T& A0, typename Vec4<R>::T& A1,
                                           uint4& A2) {
    A0.x = ph.off[0]; A0.y = ph.off[1]; A0.z = ph.off[2]; A0.w = ph.scatNext;
    A1.x = ph.d[0]; A1.y = ph.d[1]; A1.z = ph.d[2]; A1.w = idToReal<R>(ph.id);
    A2.x = packCell(ph.s & 31, ph.idx);
    A2.y = packProp(ph.w, ph.p, ph.neg) | ((uint32_t)(ph.s >> 5) << 26);
    A2.z = ph.nscat;
    A2.w = ph.nloop;
}

// ----------------------------------------------------------------- advance
// Per-launch constants of the advance kernels.
template <typename R>
struct Window {
    int keff;        // dt-steps in this launch
    R len;           // keff * dt
    R invdt;
    bool last;       // the horizon ends with this launch
    R next;          // length of the following window (0 if none)
    __device__ __forceinline__ void init(const Params<R>& P) {
        keff = P.wKeff;
        len = P.wLen;
        invdt = P.wInvdt;
        last = P.wLast != 0;
        next = P.wNext;
    }
};

// The window fields of P for its step0: keff dt-steps of length dt from
// step0, whether the horizon ends with them, and the next window's length
// (the arithmetic in the flight precision, as the kernels used to form it).
template <typename R>
__host__ __device__ inline void setWindow(Params<R>& P) {
    const int rest = P.nsteps - P.step0;
    P.wKeff = P.ksteps < rest ? P.ksteps : rest;
    P.wLen = (R)P.wKeff * P.dt;
    P.wInvdt = R(1) / P.dt;
    P.wLast = (P.step0 + P.wKeff >= P.nsteps) ? 1 : 0;
    const int after = rest - P.wKeff > 0 ? rest - P.wKeff : 0;
    P.wNext = (R)(P.ksteps < after ? P.ksteps : after) * P.dt;
}

// Face j of a subdomain: the slot's own faces, then its continuation's.
template <typename R>
__device__ __forceinline__ const FaceD<R>& faceOf(const SdomD<R>* S, int j) {
    return j < MAX_FACES ? S->f[j] : S[1].f[j - MAX_FACES];
}

// Signed distance of the phonon from a general face (SdomD::gen), from its
// frame coordinates u = idx + off.
template <typename R>
__device__ __forceinline__ R planeDist(const FaceD<R>& F, const Phn<R>& ph) {
    const R u0 = (R)ph.idx[0] + ph.off[0], u1 = (R)ph.idx[1] + ph.off[1], u2 = (R)ph.idx[2] + ph.off[2];
    return ((F.gp[0] * u0 + F.gp[1] * u1) + F.gp[2] * u2) + F.gp[3];
}

// Walker state that only the replay kernels carry.
struct NoReplay {};
template <bool REPLAY> struct ReplayState { using T = NoReplay; };
template <> struct ReplayState<true> { using T = Rng<true>; };

// Dead marker in the prop word of a slot written back in place.
constexpr uint32_t PROP_DEAD = 1u << 25;

// One phonon in flight: its state and the launch-local quantities derived
// from it. iterate() runs one loop iteration of montecarlo/problem.cpp:401-435
// (flight to the next event or to the end of the window, its tally, the
// event); finish() closes the phonon's window.
// GEN: the kernel also takes subdomains other than the Parallelepiped
// (their face planes and escape test); without it that code is compiled out.
template <typename R, bool REPLAY, bool LOG, int TM, typename IA, bool COMPACT = false, bool GEN = false>
struct Walker {
    Phn<R> ph;
    IA I;
    const SdomD<R>* S;
    R a[3], ia[3];
    R v, iv;
    R budget;
    R tnext;       // time to the next event after the window end
    int nev;       // events in this window
    int nsc;       // relaxation-time scatters in this window
    int stop;      // 0 alive, else the counter of the stop reason
    // the replay stream's position persists across events; a Philox stream
    // is set up afresh at each event from (key, phonon id, event index)
    typename ReplayState<REPLAY>::T rg;

    __device__ __forceinline__ void load(const Params<R>& P, const IA& inst, const Window<R>& W,
                                         const typename Vec4<R>::T& A0, const typename Vec4<R>::T& A1,
                                         const uint4& A2) {
        I = inst;
        unpackCell(A2.x, ph.s, ph.idx);
        ph.s |= (int)((A2.y >> 26) & 1u) << 5;
        ph.off[0] = A0.x; ph.off[1] = A0.y; ph.off[2] = A0.z; ph.scatNext = A0.w;
        ph.d[0] = A1.x; ph.d[1] = A1.y; ph.d[2] = A1.z;
        ph.id = realToId<R>(A1.w);
        ph.w = (int)(A2.y & 0xFFFFu);
        ph.p = (int)((A2.y >> 16) & 0xFFu);
        ph.neg = (A2.y >> 24) & 1u;
        ph.nscat = A2.z;
        ph.nloop = A2.w;
        if constexpr (REPLAY) rg.init(I.key0(), I.key1(), ph.id, &P);
        budget = W.len;
        S = &I.sd()[ph.s];
        reducedVel(*S, ph.d, a, ia);
        v = I.vel()[ph.w * I.np() + ph.p];
        iv = R(1) / v;
        stop = 0;
        nev = 0;
        nsc = 0;
        tnext = R(0);
    }

    __device__ __forceinline__ void pack(typename Vec4<R>::T& A0, typename Vec4<R>::T& A1, uint4& A2) const {
        packPhonon(ph, A0, A1, A2);
    }

    // returns true when the phonon's window is over (alive or stopped)
    __device__ __forceinline__ bool iterate(const Params<R>& P, const Window<R>& W) {
        // Subdomain::advect (montecarlo/subdomain.cpp:161-192): the
        // approaching face of each axis, in the reference's face order
        // (lower faces 0..2, then upper faces 3..5), against the free path;
        // strict < keeps the first of equals
        R sev = ph.scatNext;
        int face = -1;
        const bool gen = GEN && S->gen != 0;
        if (!gen) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const R dist = (-(R)ph.idx[k] - ph.off[k]) * ia[k];
                if (a[k] < R(0) && dist < sev) { sev = dist; face = k; }
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const R dist = (((R)(S->shape[k] - ph.idx[k])) - ph.off[k]) * ia[k];
                if (a[k] > R(0) && dist < sev) { sev = dist; face = k + 3; }
            }
        } else {
            // general faces: planes in frame coordinates, approached when
            // n . d < 0, at distance -(signed distance) / (n . d)
            // (montecarlo/boundary.cpp:102-110)
#pragma unroll 1
            for (int j = 0; j < S->nface; ++j) {
                const FaceD<R>& F = faceOf(S, j);
                const R nd = (F.n[0] * ph.d[0] + F.n[1] * ph.d[1]) + F.n[2] * ph.d[2];
                if (!(nd < R(0))) continue;
                const R dist = -planeDist(F, ph) / nd;
                if (dist < sev) { sev = dist; face = j; }
            }
        }
        const R tev = sev * iv;
        const bool event = tev <= budget;
        const R s = event ? sev : budget * v;
        if (gen && event) {
            // after the move: killed if it went back by more than eps or
            // left the subdomain (montecarlo/subdomain.cpp:176-189); the
            // flight is not tallied
            bool out = sev < -S->eps;
#pragma unroll 1
            for (int j = 0; j < S->nface; ++j) {
                const FaceD<R>& F = faceOf(S, j);
                const R nd = (F.n[0] * ph.d[0] + F.n[1] * ph.d[1]) + F.n[2] * ph.d[2];
                if (planeDist(F, ph) + s * nd < -S->eps) out = true;
            }
            if (out) {
                stop = C_ESCAPES;
                if (LOG) {
                    double x[3]; physPos(*S, ph, x);
                    for (int k = 0; k < 3; ++k) x[k] += (double)s * (double)ph.d[k];
                    logEvent(P, ph, ph.s, -3, ph.s, x,
                             (double)P.step0 * (double)P.dt + (double)(W.len - budget) + (double)tev,
                             ph.idx[0] * S->tstride[0] + ph.idx[1] * S->tstride[1] + ph.idx[2] * S->tstride[2]);
                }
                return true;
            }
        }
        // tally amounts per metre (montecarlo/problem.cpp:473-544)
        Tally<R, TM, IA> T;
        T.V = I;
        // field copy of this phonon (batch means), global fields only
        T.goff = (TM != TM_SHARED && I.groups() > 1) ? (long long)(ph.id % (uint32_t)I.groups()) * I.gstride() : 0;
        setFlightRows(T, I.problem(), ph.neg, iv, ph.d, ph.nscat, I.cumStep());
        const int sBefore = ph.s;
        int cellEnd = 0;
        fly<R, TM, IA, COMPACT>(ph, *S, a, ia, s, T);
        if (LOG) cellEnd = ph.idx[0] * S->tstride[0] + ph.idx[1] * S->tstride[1] + ph.idx[2] * S->tstride[2];
        ph.scatNext -= s;
        if (ph.scatNext < Lim<R>::tiny()) ph.scatNext = R(0);
        if (!event) {
            tnext = (sev - s) * iv;
            budget = R(0);
            if (!(ph.scatNext == ph.scatNext)) stop = C_BAD;
            return true;
        }
        budget -= tev;
        if (sev < -S->eps) {
            stop = C_ESCAPES;
            if (LOG) {
                double x[3]; physPos(*S, ph, x);
                logEvent(P, ph, sBefore, -3, sBefore, x, (double)P.step0 * (double)P.dt + (double)(W.len - budget),
                         cellEnd);
            }
            return true;
        }
        double xe[3];
        if (LOG) physPos(*S, ph, xe);
        Rng<REPLAY> g;
        if constexpr (REPLAY) g = rg;
        else g.init(I.key0(), I.key1(), ph.id, &P);
        g.setEvent(ph.nloop + 1);
        // the event: a relaxation scatter (kind -1) or the face's boundary
        const FaceD<R>* F = face >= 0 ? (GEN ? &faceOf(S, face) : &S->f[face]) : nullptr;
        const int kind = face >= 0 ? F->kind : -1;
        if (face >= 0 && !gen) {
            // the flight ends on the face: snap that coordinate
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (face == k) { ph.idx[k] = 0; ph.off[k] = R(0); }
                if (face == k + 3) { ph.idx[k] = S->shape[k] - 1; ph.off[k] = R(1); }
            }
        }
        // A scatter and a diffuse wall both draw a new direction: their
        // lanes make the first Philox block together and share one
        // direction draw (same words in the same order as drawIso /
        // drawAniso, so the same results), instead of each kind running
        // its own copy in turn.
        const bool draws = kind < 0 || kind == F_DIFF;
        if (draws) g.fill();
        if (kind < 0) {
            // Material::scatter (montecarlo/material.cpp:298-303)
            uint32_t x1 = g.next(), x2 = g.next();
            ph.w = searchGuided(I.wthr(), I.wguide(), I.nw(), x1);
            ph.p = searchBranch(I.pthr() + ph.w * I.np(), I.np(), x2);
        }
        if (draws) {
            // isotropic after a scatter (montecarlo/random.cpp:16-27);
            // cosine law about the inward normal at a diffuse wall
            // (montecarlo/boundary.cpp:308-312, montecarlo/random.cpp:29-44),
            // where it counts as a scatter
            R c, sn;
            const uint32_t wp = g.next();
            if (kind < 0) isoPolar(wp, c, sn);
            else anisoPolar(wp, false, c, sn);
            R sp, cp;
            sincospi_(uone<R>(g.next()), &sp, &cp);
            const R vv[3] = {sn * cp, sn * sp, c};
            if (kind < 0) { ph.d[0] = vv[0]; ph.d[1] = vv[1]; ph.d[2] = vv[2]; }
            else rotate(F->rot, vv, ph.d);
            normalize(ph.d);
            ph.nscat++;
        }
        if (kind < 0) {
            ph.scatNext = drawScatNext<R>(g, I.vt()[ph.w * I.np() + ph.p]);
            v = I.vel()[ph.w * I.np() + ph.p];
            iv = R(1) / v;
            ++nsc;
        } else if (kind == F_SPEC) {  // montecarlo/boundary.cpp:283-287
            R nd = (F->n[0] * ph.d[0] + F->n[1] * ph.d[1]) + F->n[2] * ph.d[2];
            for (int j = 0; j < 3; ++j) ph.d[j] -= R(2) * nd * F->n[j];
            normalize(ph.d);
        } else if (kind == F_ISOT) {  // montecarlo/boundary.cpp:455-460
            stop = C_ABSORBED;
        } else if (kind == F_PERI || kind == F_INTER) {
            // montecarlo/boundary.cpp:516-522 (Peri), 349-359 (Inter)
            if (GEN && kind == F_INTER && F->more != 0) {
                // several pairs: the first whose subdomain holds the
                // position, within that subdomain's escape tolerance; none
                // kills the phonon
                const FaceD<R>* cand = S[1].f + (F->more & 0xFF);
                const int nc = F->more >> 8;
                R u[3];
                for (int j = 0; j < 3; ++j) u[j] = (R)ph.idx[j] + ph.off[j];
                const FaceD<R>* pick = nullptr;
                for (int c = 0; c < nc && pick == nullptr; ++c) {
                    const FaceD<R>* C = cand + c;
                    const SdomD<R>* T = &I.sd()[C->to];
                    R u2[3];
                    rotate(C->A, u, u2);
                    for (int j = 0; j < 3; ++j) u2[j] += C->b[j];
                    bool in = true;
                    if (T->gen) {
                        // Subdomain::isInside over the target's faces
                        for (int j = 0; j < T->nface; ++j) {
                            const FaceD<R>& G = faceOf(T, j);
                            if (((G.gp[0] * u2[0] + G.gp[1] * u2[1]) + G.gp[2] * u2[2]) + G.gp[3] < -T->eps) in = false;
                        }
                    } else {
                        for (int j = 0; j < 3; ++j) {
                            const R tol = T->eps * C->n[j];
                            if (u2[j] < -tol || u2[j] > T->S[j] + tol) in = false;
                        }
                    }
                    if (in) pick = C;
                }
                F = pick;
            }
            if (F == nullptr || F->to < 0) {
                stop = C_ESCAPES;
            } else {
                if (F->tang) {
                    // same axis, tangential cells unchanged: keep the split
                    // coordinates, move onto the paired face (selects on
                    // every axis: no indexed writes into the phonon state)
                    ph.s = F->to;
                    S = &I.sd()[ph.s];
                    const int tf = F->toface;
                    const int tax = tf >= 3 ? tf - 3 : tf;
                    const bool up = tf >= 3;
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const bool on = tax == j;
                        ph.idx[j] = on ? (up ? S->shape[j] - 1 : 0) : ph.idx[j];
                        ph.off[j] = on ? (up ? R(1) : R(0)) : ph.off[j];
                    }
                } else {
                    R u[3], u2[3];
                    for (int j = 0; j < 3; ++j) u[j] = (R)ph.idx[j] + ph.off[j];
                    rotate(F->A, u, u2);
                    for (int j = 0; j < 3; ++j) u2[j] += F->b[j];
                    ph.s = F->to;
                    S = &I.sd()[ph.s];
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        if (F->toface == j) u2[j] = R(0);
                        if (F->toface == j + 3) u2[j] = S->S[j];
                    }
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        int ii = (int)floor(u2[j]);
                        ii = min(max(ii, 0), S->shape[j] - 1);
                        ph.idx[j] = ii;
                        ph.off[j] = clamp01(u2[j] - (R)ii);
                    }
                }
                if (kind == F_PERI && !F->ident) {
                    R dd[3] = {ph.d[0], ph.d[1], ph.d[2]};
                    rotate(F->Rd, dd, ph.d);
                    normalize(ph.d);
                }
            }
        }
        ++nev;
        if (LOG) logEvent(P, ph, sBefore, face, ph.s, xe, (double)P.step0 * (double)P.dt + (double)(W.len - budget),
                          cellEnd);
        ph.nloop++;
        if constexpr (REPLAY) {
            rg = g;
            if (g.exhausted()) { stop = C_REPLAY_EXHAUSTED; return true; }
        }
        if (stop) return true;
        if ((long long)ph.nscat >= I.maxscat()) { stop = C_MAXSCAT; return true; }
        if ((long long)ph.nloop >= I.maxloop()) { stop = C_MAXLOOP; return true; }
        if (nev >= MAX_EVENTS_PER_LAUNCH) { stop = C_BAD; return true; }
        reducedVel(*S, ph.d, a, ia);
        return false;
    }

    // the phonon's window is over: count its steps, events and stop
    // reason; returns true if it stays alive
    __device__ __forceinline__ bool finish(const Params<R>& P, const Window<R>& W) {
        int st;
        const bool alive = close(P, W, st);
        blkCount(C_PHONON_STEPS, (unsigned)st);
        blkCount(C_EVENTS, (unsigned)nev);
        // counted per window rather than per scatter: one block-counter add
        // per phonon instead of one per event
        if (nsc) blkCount(C_SCATTERS, (unsigned)nsc);
        return alive;
    }

    // as finish(), with the dt-steps and events of the window added to the
    // caller's per-thread sums instead of the block counters
    __device__ __forceinline__ bool finishInto(const Params<R>& P, const Window<R>& W, unsigned long long& steps,
                                               unsigned long long& events) {
        int st;
        const bool alive = close(P, W, st);
        steps += (unsigned)st;
        events += (unsigned)nev;
        if (nsc) blkCount(C_SCATTERS, (unsigned)nsc);
        return alive;
    }

    // close the window: `st` = the dt-steps the phonon was alive at the
    // start of, stop reason counted and flagged; true if it stays alive
    __device__ __forceinline__ bool close(const Params<R>& P, const Window<R>& W, int& stOut) {
        if constexpr (REPLAY) rg.save();
        int st = W.keff;
        if (stop == 0) {
            if (W.last) {
                stop = C_HORIZON;
                if (LOG) {
                    double x[3]; physPos(*S, ph, x);
                    int ce = ph.idx[0] * S->tstride[0] + ph.idx[1] * S->tstride[1] + ph.idx[2] * S->tstride[2];
                    logEvent(P, ph, ph.s, -2, ph.s, x, (double)P.nsteps * (double)P.dt, ce);
                }
            }
        } else {
            R el = W.len - budget;
            st = (int)ceil(el * W.invdt);
            st = st < 1 ? 1 : (st > W.keff ? W.keff : st);
        }
        stOut = st;
        if (stop == C_REPLAY_EXHAUSTED) atomicOr(P.status, (unsigned)S_REPLAY_EXHAUSTED);
        else if (stop == C_BAD) atomicOr(P.status, (unsigned)S_NONFINITE);
        if (stop != 0 && stop != C_REPLAY_EXHAUSTED) blkCount(stop, 1);
        return stop == 0;
    }
};

// Outcome of leanFlight.
enum { LEAN_EVENT = 0, LEAN_ALIVE = 1, LEAN_BAD = 2 };

// One window of a phonon whose next event lies beyond the window end, in a
// single-instance launch with a shared field whose subdomains all tally
// along axis K (a 1-D field). It is Walker::load, the first
// Walker::iterate and Walker::close of such a phonon, operation for
// operation (the same arithmetic in the same order, so the same results),
// without the walker's event handling, loop and bookkeeping. Returns
// LEAN_EVENT, having changed nothing, if the phonon does meet an event in
// the window (the caller then runs the walker); otherwise the flight is
// tallied, the state packed back into A0..A2, *tnext set to the time from
// the window end to the next event, and LEAN_ALIVE returned (LEAN_BAD for a
// non-finite free path, which the caller counts as the walker would).
template <typename R, int K, typename IA, bool SPLIT = false>
__device__ __forceinline__ int leanFlight(const IA& I, const Window<R>& W, typename Vec4<R>::T& A0,
                                          typename Vec4<R>::T& A1, uint4& A2, R& tnext) {
    Phn<R> ph;
    unpackCell(A2.x, ph.s, ph.idx);
        ph.s |= (int)((A2.y >> 26) & 1u) << 5;
    ph.off[0] = A0.x; ph.off[1] = A0.y; ph.off[2] = A0.z; ph.scatNext = A0.w;
    ph.d[0] = A1.x; ph.d[1] = A1.y; ph.d[2] = A1.z;
    ph.id = realToId<R>(A1.w);
    ph.w = (int)(A2.y & 0xFFFFu);
    ph.p = (int)((A2.y >> 16) & 0xFFu);
    ph.neg = (A2.y >> 24) & 1u;
    ph.nscat = A2.z;
    ph.nloop = A2.w;
    const SdomD<R>& S = I.sd()[ph.s];
    R a[3], ia[3];
    reducedVel(S, ph.d, a, ia);
    const R v = I.vel()[ph.w * I.np() + ph.p];
    const R iv = R(1) / v;
    R sev = ph.scatNext;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const R dist = (-(R)ph.idx[k] - ph.off[k]) * ia[k];
        if (a[k] < R(0) && dist < sev) sev = dist;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const R dist = (((R)(S.shape[k] - ph.idx[k])) - ph.off[k]) * ia[k];
        if (a[k] > R(0) && dist < sev) sev = dist;
    }
    if (sev * iv <= W.len) return LEAN_EVENT;
    const R s = W.len * v;
    Tally<R, TM_SHARED, IA, SPLIT> T;
    T.V = I;
    T.goff = 0;
    setFlightRows(T, I.problem(), ph.neg, iv, ph.d, ph.nscat, I.cumStep());
    fly1d<R, TM_SHARED, IA, SPLIT>(ph, S, a, ia, s, T, K);
    ph.scatNext -= s;
    if (ph.scatNext < Lim<R>::tiny()) ph.scatNext = R(0);
    tnext = (sev - s) * iv;
    if (!(ph.scatNext == ph.scatNext)) return LEAN_BAD;
    packPhonon(ph, A0, A1, A2);
    return LEAN_ALIVE;
}

// Add the block's counters to the launch counters (after a barrier).
__device__ __forceinline__ void flushCounts(unsigned long long* counters) {
    for (int q = threadIdx.x; q < C_NCOUNTERS; q += blockDim.x)
        if (g_blk.cnt[q]) atomicAdd(&counters[q], g_blk.cnt[q]);
}

}  // namespace mcg
