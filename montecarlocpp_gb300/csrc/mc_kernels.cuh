// mc_kernels.cuh -- sm_103a kernels of the phonon particle-advance hot path.
//
// One thread owns one phonon. A launch advances every live phonon through a
// time window of K dt-steps, event by event (montecarlo/problem.cpp:401-435):
// nearest approaching face versus the free path (Subdomain::advect,
// montecarlo/subdomain.cpp:161-192), the flight tallied cell by cell
// (Field::accumulate, montecarlo/field.cpp:160-288), then the boundary event
// or the relaxation-time scatter (Walker, mc_walker.cuh).
//
//   k_emit / k_emit_batch   emission (event 0 of each phonon's stream)
//   k_advance               static: each block streams its region of the
//                           state through shared memory by bulk copies (one
//                           producer warp), one phonon per consumer thread;
//                           survivors go to the region's two ends in the
//                           other half (next event inside the next window
//                           at the front)
//   k_advance_dyn           dynamic: warps refill idle lanes from a
//                           block-owned queue; state written back in place
//   k_advance_batch         dynamic, over many instances in one launch
//   k_compact               stream compaction of dead slots
//   k_difprefix             global difference arrays -> field (batched)
#pragma once

#include "mc_async.cuh"
#include "mc_walker.cuh"

namespace mcg {

// One constant table into shared memory: its 16-byte-aligned body by a
// bulk copy (the TMA engine, completing on a block mbarrier), the rest
// element by element by all threads. A table whose source or destination
// is not 16-byte aligned is copied by the threads whole.
template <typename T>
struct TableCopy {
    T* dst;
    const T* src;
    int n;
    uint32_t body;  // bytes the bulk copy takes
    __device__ __forceinline__ TableCopy(T* d, const T* s, int count) : dst(d), src(s), n(count) {
        const bool aligned = MC_TABLE_BULK && count > 0 && (((uintptr_t)s | (uintptr_t)smemAddr(d)) & 15) == 0;
        body = aligned ? (uint32_t)((sizeof(T) * (size_t)count) & ~(size_t)15) : 0u;
    }
    // thread 0: the bulk copy, after the barrier expects its bytes
    __device__ __forceinline__ void issue(uint64_t* bar) const {
        if (body) bulkLoad(dst, src, body, bar);
    }
    __device__ __forceinline__ void rest() const {
        for (int i = (int)(body / sizeof(T)) + (int)threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
    }
};

// A bounded wait on the table copies of stageTables (they complete in
// microseconds; the limit only keeps a broken copy from hanging the block)
constexpr uint64_t TABLE_COPY_WAIT_NS = 1000000000ull;

// Instance descriptor of a single-instance launch, around the tables it
// staged in shared memory. The tables go in by bulk copies, so a block's
// staging costs about one round trip rather than one per loop iteration.
template <typename R, int TM>
__device__ __forceinline__ InstD<R>* stageTables(const Params<R>& P, unsigned char* smraw) {
    __shared__ uint64_t barTab;
    const int nt = P.nw * P.np;
    const int nsdShared = P.nsd;
    const SmemLayout L = singleLayout<R>(P.nw, P.np, P.nsd, P.rows, P.cols, TM == TM_SHARED, false, !P.tabGlobal);
    R* vel = reinterpret_cast<R*>(smraw + L.vel);
    R* vt = P.tabGlobal ? const_cast<R*>(P.vt) : reinterpret_cast<R*>(smraw + L.vt);
    unsigned long long* wthr = reinterpret_cast<unsigned long long*>(smraw + L.wthr);
    uint16_t* wguide = P.tabGlobal ? const_cast<uint16_t*>(P.wguide) : reinterpret_cast<uint16_t*>(smraw + L.guide);
    long long* tal = reinterpret_cast<long long*>(smraw + L.tal);
    InstD<R>* I = reinterpret_cast<InstD<R>*>(smraw + L.inst);
    const TableCopy<R> cVel(vel, P.vel, nt);
    const TableCopy<R> cVt(vt, P.vt, P.tabGlobal ? 0 : nt);
    const TableCopy<uint16_t> cGuide(wguide, P.wguide, P.tabGlobal ? 0 : GUIDE);
    const TableCopy<unsigned long long> cWthr(wthr, P.wthr, P.nw);
    const TableCopy<uint32_t> cSd(reinterpret_cast<uint32_t*>(smraw + L.sd), reinterpret_cast<const uint32_t*>(P.sd),
                                  (int)(sizeof(SdomD<R>) * nsdShared / 4));
    const SdomD<R>* sd = nsdShared ? reinterpret_cast<const SdomD<R>*>(smraw + L.sd) : P.sd;
    if (threadIdx.x == 0) {
        mbarInit(&barTab, 1);
        mbarInitFence();
        mbarArriveExpectTx(&barTab, cVel.body + cVt.body + cGuide.body + cWthr.body + cSd.body);
        cVel.issue(&barTab);
        cVt.issue(&barTab);
        cGuide.issue(&barTab);
        cWthr.issue(&barTab);
        cSd.issue(&barTab);
    }
    cVel.rest();
    cVt.rest();
    cGuide.rest();
    cWthr.rest();
    cSd.rest();
    if (TM == TM_SHARED) {
        const int nz = (int)talEntries(P.rows, P.cols);
        for (int i = threadIdx.x; i < nz; i += blockDim.x) tal[i] = 0;
        if (P.smSplit) {
            unsigned* sp = reinterpret_cast<unsigned*>(smraw + P.smSplit);
            for (int i = threadIdx.x; i < 2 * nz; i += blockDim.x) sp[i] = 0u;
        }
    }
    if (threadIdx.x == 0) {
        I->vel = vel; I->vt = vt; I->wthr = wthr; I->wguide = wguide; I->pthr = P.pthr;
        I->fwthr = P.fwthr; I->fpthr = P.fpthr;
        I->sd = sd; I->em = P.em; I->emitCdf = P.emitCdf;
        I->nw = P.nw; I->np = P.np; I->nem = P.nem; I->nsd = P.nsd;
        I->problem = P.problem; I->rows = P.rows; I->cols = P.cols; I->inst = 0; I->cumStep = P.cumStep;
        I->maxscat = P.maxscat; I->maxloop = P.maxloop;
        I->slot0 = 0; I->nemit = P.nemit;
        I->key0 = P.key0; I->key1 = P.key1;
        I->tal = TM == TM_SHARED ? tal : nullptr;
        I->dif = TM == TM_SHARED ? tal + (size_t)talStride(P.rows) * P.cols : nullptr;
        I->tally = P.tally; I->gdif = nullptr; I->csum = P.csum;
        I->groups = 1; I->gstride = 0; I->flags = 0;
        for (int r = 0; r < 4; ++r) { I->tqinv[r] = P.tqinv[r]; I->tq[r] = P.tq[r]; }
    }
    __syncthreads();  // the barrier's initialisation seen by every thread
    if (!mbarWait(&barTab, 0u, TABLE_COPY_WAIT_NS)) atomicOr(P.status, (unsigned)S_TIMEOUT);
    return I;
}

// Flush the block's shared fixed-point field into `dst` (rows x cols,
// column-major) as FP64 atomics and clear it: first the difference array
// is prefix-summed into the cells, then every non-zero cell is added and
// summed per row into the block checksums (the field holds every flight
// amount that did not go to g_blk.csum directly). Both shared arrays are
// cell-major with talStride(rows) words per cell; dst is rows x cols
// column-major. All threads, after a barrier.
template <typename R>
__device__ __forceinline__ void flushSharedField(const InstD<R>& I, double* dst) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int rows = I.rows, st = talStride(rows);
    for (int r = warp; r < rows; r += nwarps) {
        long long carry = 0;
        for (int c0 = 0; c0 < I.cols; c0 += 32) {
            const int c = c0 + lane;
            long long x = c < I.cols ? I.dif[c * st + r] : 0;
            if (c < I.cols) I.dif[c * st + r] = 0;
            for (int o = 1; o < 32; o <<= 1) {
                long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= o) x += y;
            }
            x += carry;
            if (c < I.cols) I.tal[c * st + r] += x;
            carry = __shfl_sync(0xFFFFFFFFu, x, 31);
        }
        if (lane == 0) I.dif[I.cols * st + r] = 0;
    }
    __syncthreads();
    long long part[4] = {0, 0, 0, 0};
    const int tot = rows * I.cols;
    for (int q = threadIdx.x; q < tot; q += blockDim.x) {
        const int c = q / rows, r = q - c * rows;
        const long long x = I.tal[c * st + r];
        if (x != 0) {
            const int k0 = rowClass(I.problem, r);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k == k0) part[k] += x;
            atomicAdd(&dst[q], (double)x * I.tq[k0]);
            I.tal[c * st + r] = 0;
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        long long x = part[r];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if (lane == 0 && x != 0) sharedAdd64(&g_blk.csum[r], x);
    }
}

// End of a single-instance launch: the shared field flushed into the global
// one, the block checksums and counters added to the launch's.
template <typename R, int TM>
__device__ __forceinline__ void closeBlock(const Params<R>& P, const InstD<R>& I) {
    __syncthreads();
    if (TM == TM_SHARED && P.smSplit) {
        // fold the lean flights' carry-free field into the 64-bit one
        const int nz = (int)talEntries(P.rows, P.cols);
        const unsigned char* base = reinterpret_cast<const unsigned char*>(I.tal) - P.smTal;
        const unsigned* lo = reinterpret_cast<const unsigned*>(base + P.smSplit);
        const int* hi = reinterpret_cast<const int*>(lo) + nz;
        for (int e = threadIdx.x; e < nz; e += blockDim.x) {
            const long long v = (long long)hi[e] * (1LL << SPLIT_LOW_BITS) + (long long)lo[e];
            if (v != 0) I.tal[e] += v;
        }
        __syncthreads();
    }
    if (TM == TM_SHARED) flushSharedField<R>(I, P.tally);
    __syncthreads();
    if ((int)threadIdx.x < rowClasses(I.problem, I.rows) && g_blk.csum[threadIdx.x] != 0)
        atomicAdd(&P.csum[threadIdx.x], (double)g_blk.csum[threadIdx.x] * I.tq[threadIdx.x]);
    flushCounts(P.counters);
}

// -------------------------------------------------------------- emission
template <typename R, bool REPLAY>
__global__ void __launch_bounds__(256) k_emit(Params<R> P) {
    __shared__ InstD<R> I;
    if (threadIdx.x == 0) {
        I.fwthr = P.fwthr; I.fpthr = P.fpthr; I.vt = P.vt; I.sd = P.sd; I.em = P.em; I.emitCdf = P.emitCdf;
        I.nw = P.nw; I.np = P.np; I.nem = P.nem;
    }
    __syncthreads();
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.nemit) return;
    // static schedule: the phonons of each block region start at its front
    if (P.regIn != nullptr && n % P.regCap == 0)
        P.regIn[2 * (n / P.regCap)] = (unsigned)min(P.regCap, P.nemit - n);
    Rng<REPLAY> g;
    g.init(P.key0, P.key1, (uint32_t)n, &P);
    Phn<R> ph;
    emitOne<R>(I, n, g, ph);
    if (REPLAY) {
        g.save();
        if (g.exhausted()) atomicOr(P.status, (unsigned)S_REPLAY_EXHAUSTED);
    }
    typename Vec4<R>::T a, b;
    uint4 c;
    packPhonon(ph, a, b, c);
    st4(P.P0out + n, a);
    st4(P.P1out + n, b);
    __stcs(P.P2out + n, c);
}

// Instance owning a batch slot: the last i with islot[i] <= n.
__device__ __forceinline__ int instanceOf(const long long* islot, int ninst, long long n) {
    int lo = 0, hi = ninst;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (islot[mid + 1] <= n) lo = mid + 1; else hi = mid;
    }
    return lo < ninst ? lo : ninst - 1;
}

// Phonon id of slot `local` of an instance whose n phonons are split into
// G field copies stored one after the other: copy g holds the ids equal to
// g mod G (the first n % G copies one more than the others), so that every
// copy samples all emitters alike.
__host__ __device__ __forceinline__ long long groupedId(long long local, long long n, int G) {
    if (G <= 1) return local;
    const long long q = n / G, rem = n % G;
    long long g, j;
    if (local < rem * (q + 1)) {
        g = local / (q + 1);
        j = local - g * (q + 1);
    } else {
        const long long t = local - rem * (q + 1);
        g = rem + t / q;
        j = t - (g - rem) * q;
    }
    return j * G + g;
}

// Emission of every instance of a launch: thread n takes phonon n - islot[i]
// of the instance i whose range [islot[i], islot[i + 1]) holds n, writes it
// to that instance's state slot I.slot0 + (n - islot[i]) (a batch lays its
// instances out back to back, so that slot is n; a served round sits in the
// slots it was given), and its phonon id follows by groupedId.
template <typename R>
__global__ void __launch_bounds__(256) k_emit_batch(Params<R> P) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= (long long)P.cap) return;
    const int i = instanceOf(P.islot, P.ninst, n);
    const InstD<R>& I = P.insts[i];
    const long long local = n - P.islot[i];
    const long long slot = I.slot0 + local;
    const long long id = groupedId(local, I.nemit, I.groups);
    Rng<false> g;
    g.init(I.key0, I.key1, (uint32_t)id, &P);
    Phn<R> ph;
    emitOne<R>(I, id, g, ph);
    typename Vec4<R>::T a, b;
    uint4 c;
    packPhonon(ph, a, b, c);
    st4(P.P0out + slot, a);
    st4(P.P1out + slot, b);
    __stcs(P.P2out + slot, c);
}

// ----------------------------------------------------------------- advance
// Static kernel: a persistent, warp-specialised stream over the block's
// region of the state.
//
// Block b owns slots [b C, (b + 1) C) of both halves of the state (C =
// regCap). Its live phonons sit at the two ends of its region in the input
// half: regIn[2b] at the front (their next event falls inside this
// window), regIn[2b + 1] at the back (no event in it). The block's last
// warp is the producer: one lane walks the front range, then the back
// range, in tiles of T = blockDim.x - 32 slots and issues cp.async.bulk
// copies of each tile (48 B per phonon in FP32: three 16-byte words, one
// copy per word array) into one of STATIC_STAGES shared-memory stages,
// completing on the stage's mbarrier. The other T threads (the consumers)
// each take one phonon of a tile out of the stage, release the stage at
// once (so the next copy overlaps their work), advance the phonon through
// the window, and write the survivors to the block's region of the output
// half: phonons whose next event falls inside the next window from the
// front, the others from the back, positions taken from two shared-memory
// counters per warp ballot. Stopped phonons are dropped. The warps of a
// block never wait for one another, a tile holds phonons of one kind (events
// or plain flights), and no global atomic is involved. Step and
// event counts are summed per thread and added to the block's counters
// once, at the end.
constexpr int STATIC_STAGES = MC_STATIC_STAGES;
constexpr int STATIC_PRODUCER_THREADS = 32;
// consumer threads per block at most (the default block size) and threads
// per block at most, by flight precision
template <typename R>
__host__ __device__ constexpr int staticConsumers() {
    return sizeof(R) == 4 ? MC_STATIC_CONSUMERS : MC_STATIC_CONSUMERS_F64;
}
template <typename R>
__host__ __device__ constexpr int staticMaxThreads() {
    return staticConsumers<R>() + STATIC_PRODUCER_THREADS;
}
constexpr unsigned STATIC_END = 0xFFFFFFFFu;  // stage marker: no more tiles
constexpr unsigned STATIC_BACK = 1u << 30;    // stage tag: a tile of the back range
// bounded waits: a bulk copy lands within microseconds; the producer may
// wait for consumers in the middle of a long window much longer
constexpr uint64_t STATIC_COPY_WAIT_NS = 2000000000ull;
constexpr uint64_t STATIC_STAGE_WAIT_NS = 60000000000ull;

template <typename R>
__host__ __device__ inline size_t staticStageBytes(int tile) {
    return (size_t)tile * (2 * sizeof(typename Vec4<R>::T) + sizeof(uint4));
}
// offset of the first stage after the single-instance layout
__host__ __device__ inline size_t staticStageOffset(size_t layoutTotal) {
    return (layoutTotal + 127) & ~(size_t)127;
}

// The shared-memory offsets of a single-instance launch into P (host).
template <typename R>
inline void setSingleLayout(Params<R>& P, const SmemLayout& L) {
    P.smVt = (int)L.vt;
    P.smWthr = (int)L.wthr;
    P.smGuide = (int)L.guide;
    P.smSd = (int)L.sd;
    P.smTal = (int)L.tal;
    P.smSplit = (int)L.split;
    P.smStage = (int)staticStageOffset(L.total);
}

// LEAN = K >= 0 (single-instance, shared field, every subdomain tallying
// along axis K, no replay, no log): the phonons of the back range, whose
// next event lies beyond this window, take leanFlight; the walker runs for
// the front range, for a back-range phonon that does meet an event, and in
// the window that ends the horizon.
template <typename R, bool REPLAY, bool LOG, int TM, int LEAN, bool GEN = false>
__global__ void __launch_bounds__(staticMaxThreads<R>(), sizeof(R) == 4 ? MC_MIN_BLOCKS_STATIC_F32 : 2)
k_advance(Params<R> P) {
    static_assert(LEAN < 0 || (!REPLAY && !LOG && TM == TM_SHARED), "the lean flight needs a plain shared-field launch");
    using V4 = typename Vec4<R>::T;
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ uint64_t barFull[STATIC_STAGES], barEmpty[STATIC_STAGES];
    __shared__ unsigned sCnt[STATIC_STAGES];
    __shared__ unsigned sOut[2];
    __shared__ int sStop;
    const int T = (int)blockDim.x - STATIC_PRODUCER_THREADS;
    const int nCw = T >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if constexpr (MC_PDL != 0) gridDepTrigger();
    InstD<R>* I = stageTables<R, TM>(P, smraw);
    ParamView<R, TM> V;
    V.init(P, smraw);
    unsigned char* stage0 = smraw + P.smStage;
    const size_t sbytes = staticStageBytes<R>(T);
    const long long C = P.regCap;
    const long long rbase = (long long)blockIdx.x * C;
    blkZero();
    if (threadIdx.x == 0) {
        for (int s = 0; s < STATIC_STAGES; ++s) {
            mbarInit(&barFull[s], 1);
            mbarInit(&barEmpty[s], (uint32_t)nCw);
        }
        sStop = 0;
        sOut[0] = sOut[1] = 0u;
        mbarInitFence();
    }
    __syncthreads();
    // the tables are constant; the state, the region counts and the field
    // belong to the previous launch until it has completed
    if constexpr (MC_PDL != 0) gridDepWait();

    if (warp == nCw) {
        // ---------------------------------------------------- producer
        if (lane == 0) {
            // the input counts, clamped to the region
            const unsigned long long nF = min((unsigned long long)P.regIn[2 * blockIdx.x], (unsigned long long)C);
            const unsigned long long nB =
                min((unsigned long long)P.regIn[2 * blockIdx.x + 1], (unsigned long long)C - nF);
            const long long tF = ((long long)nF + T - 1) / T;
            const long long tB = ((long long)nB + T - 1) / T;
            const uint32_t perPhonon = (uint32_t)(2 * sizeof(V4) + sizeof(uint4));
            long long jF = 0, jB = 0;
            int j = 0;
            for (;; ++j) {
                const int s = j % STATIC_STAGES;
                const uint32_t use = (uint32_t)(j / STATIC_STAGES);
                if (use > 0 && !mbarWait(&barEmpty[s], (use - 1) & 1u, STATIC_STAGE_WAIT_NS, &sStop)) {
                    atomicOr(P.status, (unsigned)S_TIMEOUT);
                    sStop = 1;
                    break;
                }
                if (j >= tF + tB) {
                    sCnt[s] = STATIC_END;
                    mbarArrive(&barFull[s]);
                    ++j;
                    break;
                }
                // the front range (event tiles) first: measured 12% faster
                // over a whole horizon than front tiles spread evenly among
                // the back ones
                long long src;
                unsigned cnt;
                const bool front = jF < tF;
                if (front) {
                    src = rbase + jF * T;
                    cnt = (unsigned)min((long long)T, (long long)nF - jF * T);
                    ++jF;
                } else {
                    src = rbase + C - (long long)nB + jB * T;
                    cnt = (unsigned)min((long long)T, (long long)nB - jB * T);
                    ++jB;
                }
                sCnt[s] = cnt | (front ? 0u : STATIC_BACK);
                unsigned char* st = stage0 + (size_t)s * sbytes;
                mbarArriveExpectTx(&barFull[s], cnt * perPhonon);
                bulkLoad(st, P.P0in + src, cnt * (uint32_t)sizeof(V4), &barFull[s]);
                bulkLoad(st + (size_t)T * sizeof(V4), P.P1in + src, cnt * (uint32_t)sizeof(V4), &barFull[s]);
                bulkLoad(st + (size_t)T * 2 * sizeof(V4), P.P2in + src, cnt * (uint32_t)sizeof(uint4), &barFull[s]);
            }
            // every copy this block issued has landed before it exits
            const int issued = j;
            for (int s = 0; s < STATIC_STAGES && s < issued; ++s) {
                const int last = issued - 1 - ((issued - 1 - s) % STATIC_STAGES);
                if (!mbarWait(&barFull[s], (uint32_t)(last / STATIC_STAGES) & 1u, STATIC_COPY_WAIT_NS))
                    atomicOr(P.status, (unsigned)S_TIMEOUT);
            }
        }
    } else {
        // ---------------------------------------------------- consumers
        Window<R> W;
        W.init(P);
        const unsigned lt = (1u << lane) - 1u;
        unsigned long long nSteps = 0, nEvents = 0;
        for (int j = 0;; ++j) {
            const int s = j % STATIC_STAGES;
            const uint32_t use = (uint32_t)(j / STATIC_STAGES);
            if (!mbarWait(&barFull[s], use & 1u, STATIC_COPY_WAIT_NS, &sStop)) {
                if (lane == 0) { atomicOr(P.status, (unsigned)S_TIMEOUT); sStop = 1; }
                break;
            }
            const unsigned tag = sCnt[s];
            if (tag == STATIC_END) break;
            const unsigned cnt = tag & ~STATIC_BACK;
            const bool back = (tag & STATIC_BACK) != 0;
            const int i = threadIdx.x;
            V4 A0, A1;
            uint4 A2;
            const bool have = i < (int)cnt;
            if (have) {
                const unsigned char* st = stage0 + (size_t)s * sbytes;
                A0 = reinterpret_cast<const V4*>(st)[i];
                A1 = reinterpret_cast<const V4*>(st + (size_t)T * sizeof(V4))[i];
                A2 = reinterpret_cast<const uint4*>(st + (size_t)T * 2 * sizeof(V4))[i];
            }
            __syncwarp();
            if (lane == 0) mbarArrive(&barEmpty[s]);
            if (__ballot_sync(0xFFFFFFFFu, have) == 0) continue;
            bool alive = false, soon = false;
            int lean = LEAN_EVENT;
            if constexpr (LEAN >= 0) {
                if (have && back && !W.last) {
                    R tnext;
                    lean = leanFlight<R, (LEAN >= 0 ? LEAN : 0), ParamView<R, TM>, (sizeof(R) == 4)>(V, W, A0, A1,
                                                                                                  A2, tnext);
                    if (lean != LEAN_EVENT) {
                        nSteps += (unsigned)W.keff;
                        alive = lean == LEAN_ALIVE;
                        soon = tnext < W.next;
                        if (!alive) {  // as Walker::close for a non-finite state
                            blkCount(C_BAD, 1);
                            atomicOr(P.status, (unsigned)S_NONFINITE);
                        }
                    }
                }
            }
            if (have && lean == LEAN_EVENT) {
                Walker<R, REPLAY, LOG, TM, ParamView<R, TM>, true, GEN> wk;
                wk.load(P, V, W, A0, A1, A2);
                while (!wk.iterate(P, W)) {}
                alive = wk.finishInto(P, W, nSteps, nEvents);
                soon = wk.tnext < W.next;
                if (alive) wk.pack(A0, A1, A2);
            }
            const unsigned mf = __ballot_sync(0xFFFFFFFFu, alive && soon);
            const unsigned mb = __ballot_sync(0xFFFFFFFFu, alive && !soon);
            unsigned bf = 0, bb = 0;
            if (lane == 0) {
                if (mf) bf = atomicAdd(&sOut[0], (unsigned)__popc(mf));
                if (mb) bb = atomicAdd(&sOut[1], (unsigned)__popc(mb));
            }
            bf = __shfl_sync(0xFFFFFFFFu, bf, 0);
            bb = __shfl_sync(0xFFFFFFFFu, bb, 0);
            if (alive) {
                const long long o = soon ? rbase + bf + __popc(mf & lt) : rbase + C - 1 - (bb + __popc(mb & lt));
                st4(P.P0out + o, A0);
                st4(P.P1out + o, A1);
                __stcs(P.P2out + o, A2);
            }
        }
        // per-thread sums -> block counters
        for (int o = 16; o > 0; o >>= 1) {
            nSteps += __shfl_down_sync(0xFFFFFFFFu, nSteps, o);
            nEvents += __shfl_down_sync(0xFFFFFFFFu, nEvents, o);
        }
        if (lane == 0) {
            if (nSteps) sharedAdd64(&g_blk.cnt[C_PHONON_STEPS], nSteps);
            if (nEvents) sharedAdd64(&g_blk.cnt[C_EVENTS], nEvents);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // a block that gave up leaves nothing for later launches
        const bool ok = *reinterpret_cast<volatile int*>(&sStop) == 0;
        P.regOut[2 * blockIdx.x] = ok ? sOut[0] : 0u;
        P.regOut[2 * blockIdx.x + 1] = ok ? sOut[1] : 0u;
    }
    closeBlock<R, TM>(P, *I);
}

// Dynamic schedule shared by the single-instance and batched kernels: the
// warps of a block take slots of [qbeg, qend) from the counter *qnext
// (shared for a block's own chunk, global for a batched segment); each warp
// keeps its lanes busy by refilling finished lanes whenever at least REFILL
// of them are idle, so a long phonon no longer holds up its warp. Survivors
// are written back in place; dead slots get PROP_DEAD (skipped until the
// host compacts). Refilling as soon as one lane is idle measured fastest on
// the film over a whole horizon (90.2 ms against 93.1 at 4, 98.3 at 8, 109
// at 16): an idle lane costs more than the refill's shared atomic and loads.
#ifndef MC_REFILL
#define MC_REFILL 1
#endif
constexpr int REFILL = MC_REFILL;

// cap (with the block's shared counter `claimed`): a block stops claiming
// once it holds that many slots (0: no limit).
template <typename R, bool REPLAY, bool LOG, int TM, typename IA, bool GEN = false>
__device__ __forceinline__ void dynamicLoop(const Params<R>& P, unsigned long long* qnext,
                                            unsigned long long qbeg, unsigned long long qend,
                                            const IA& I, const Window<R>& W,
                                            unsigned long long cap = 0, unsigned long long* claimed = nullptr) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    Walker<R, REPLAY, LOG, TM, IA, false, GEN> wk;
    bool have = false;
    unsigned long long slot = 0;
    bool drained = qbeg >= qend;
    uint32_t alive = 0;
    for (int guard = 0; guard < (1 << 30); ++guard) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !have);
        if (!drained && (idle == 0xFFFFFFFFu || __popc(idle) >= REFILL)) {
            unsigned long long b = 0;
            if (lane == 0) {
                const bool full = cap != 0 && atomicAdd(claimed, (unsigned long long)__popc(idle)) >= cap;
                b = full ? qend : qbeg + atomicAdd(qnext, (unsigned long long)__popc(idle));
            }
            b = __shfl_sync(0xFFFFFFFFu, b, 0);
            if (b + __popc(idle) >= qend) drained = true;
            if (!have) {
                const unsigned long long my = b + __popc(idle & lt);
                if (my < qend) {
                    // all three words at once (one memory round trip, not
                    // two); a dead slot's position and direction go unused
                    typename Vec4<R>::T A0, A1;
                    const uint4 A2 = __ldcs(P.P2in + my);
                    ld4(P.P0in + my, A0);
                    ld4(P.P1in + my, A1);
                    if (!(A2.y & PROP_DEAD)) {
                        wk.load(P, I, W, A0, A1, A2);
                        have = true;
                        slot = my;
                    }
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, have) == 0) {
            if (drained) break;
            continue;
        }
        if (have && wk.iterate(P, W)) {
            typename Vec4<R>::T A0, A1;
            uint4 A2;
            if (wk.finish(P, W)) {
                wk.pack(A0, A1, A2);
                st4(P.P0out + slot, A0);
                st4(P.P1out + slot, A1);
                __stcs(P.P2out + slot, A2);
                ++alive;
            } else if (!W.last) {
                // no later launch reads the slots after the horizon
                A2.x = 0u; A2.y = PROP_DEAD; A2.z = 0u; A2.w = 0u;
                __stcs(P.P2out + slot, A2);
            }
            have = false;
        }
    }
    // survivors: the host compacts when many slots are dead
    unsigned long long x = alive;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
    if (lane == 0 && x) atomicAdd(&P.live_out[0], x);
}

// Every block claims slots of [0, n) from the launch-wide counter
// P.qglobal, so blocks (and the SMs they run on) keep taking phonons until
// none is left and finish within about one phonon's work of one another;
// without it (short windows), block b owns the live slots [b C, (b + 1) C).
// In FP64 flight the tally quantum bounds a block's sum for C phonons with
// 4x headroom, so a block claims at most 2 C slots.
template <typename R, bool REPLAY, bool LOG, int TM, bool GEN = false>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance_dyn(Params<R> P) {
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ unsigned long long qnext, claimed;
    InstD<R>* I = stageTables<R, TM>(P, smraw);
    blkZero();
    if (threadIdx.x == 0) qnext = claimed = 0;
    __syncthreads();
    Window<R> W;
    W.init(P);
    const unsigned long long n = P.live_in[0];
    const unsigned long long chunk = (n + gridDim.x - 1) / gridDim.x;
    unsigned long long* q = &qnext;
    unsigned long long qbeg = 0, qend = n, cap = 0;
    if (P.qglobal == nullptr) {
        qbeg = min((unsigned long long)blockIdx.x * chunk, n);
        qend = min(qbeg + chunk, n);
    } else {
        q = P.qglobal;
        if (sizeof(R) == 8) cap = 2 * chunk;
    }
    ParamView<R, TM> V;
    V.init(P, smraw);
    dynamicLoop<R, REPLAY, LOG, TM, ParamView<R, TM>, GEN>(P, q, qbeg, qend, V, W, cap, &claimed);
    closeBlock<R, TM>(P, *I);
}

// The current instance of a batched block, staged in shared memory: its
// descriptor, velocity and scatter tables, and (flags permitting) its
// subdomain images and a zeroed fixed-point field with difference array.
template <typename R>
__device__ __forceinline__ void stageInstance(const Params<R>& P, int inst, unsigned char* smraw,
                                              const BatchSmem& L) {
    const InstD<R>& G = P.insts[inst];
    InstD<R>* I = reinterpret_cast<InstD<R>*>(smraw + L.inst);
    R* vel = reinterpret_cast<R*>(smraw + L.vel);
    R* vt = reinterpret_cast<R*>(smraw + L.vt);
    unsigned long long* wthr = reinterpret_cast<unsigned long long*>(smraw + L.wthr);
    uint16_t* wguide = reinterpret_cast<uint16_t*>(smraw + L.guide);
    long long* tal = reinterpret_cast<long long*>(smraw + L.tal);
    const int nt = G.nw * G.np;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        vel[i] = G.vel[i];
        vt[i] = G.vt[i];
    }
    for (int i = threadIdx.x; i < G.nw; i += blockDim.x) wthr[i] = G.wthr[i];
    for (int i = threadIdx.x; i < GUIDE; i += blockDim.x) wguide[i] = G.wguide[i];
    const bool sdS = (G.flags & IF_SD_SHARED) != 0;
    if (sdS) {
        const int nw4 = (int)(sizeof(SdomD<R>) * (size_t)G.nsd / 4);
        uint32_t* dst = reinterpret_cast<uint32_t*>(smraw + L.sd);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(G.sd);
        for (int i = threadIdx.x; i < nw4; i += blockDim.x) dst[i] = src[i];
    }
    const bool talS = (G.flags & IF_TAL_SHARED) != 0;
    if (talS) {
        const int nz = (int)talEntries(G.rows, G.cols);
        for (int i = threadIdx.x; i < nz; i += blockDim.x) tal[i] = 0;
    }
    if (threadIdx.x == 0) {
        *I = G;
        I->vel = vel; I->vt = vt; I->wthr = wthr; I->wguide = wguide;
        if (sdS) I->sd = reinterpret_cast<const SdomD<R>*>(smraw + L.sd);
        I->tal = talS ? tal : nullptr;
        I->dif = talS ? tal + (size_t)talStride(G.rows) * G.cols : nullptr;
    }
}

// End of a batched block's binding to (instance, group): the shared field,
// if any, flushed into field copy `group`, and the binding's checksums added
// to the copy's. All threads, after the binding's barrier.
template <typename R>
__device__ __forceinline__ void flushBinding(const InstD<R>& I, int group) {
    if (I.tal != nullptr) flushSharedField<R>(I, I.tally + (long long)group * I.gstride);
    __syncthreads();
    if (threadIdx.x < 4) {
        const long long x = g_blk.csum[threadIdx.x];
        if ((int)threadIdx.x < rowClasses(I.problem, I.rows) && x != 0)
            atomicAdd(&I.csum[4 * group + threadIdx.x], (double)x * I.tq[threadIdx.x]);
        g_blk.csum[threadIdx.x] = 0;
    }
}

// Batched kernel: every block binds to one work segment at a time (one
// instance, one field copy), stages that instance in shared memory and runs
// the dynamic schedule over the segment's slots together with every other
// block bound to it; when the segment has no slots left the block flushes
// its field and moves on to the next segment with work, so that a few
// expensive instances end up spread over the whole GPU. A block starts on
// segment home[block] (the host spreads blocks over segments by size).
// TM: the field mode of every instance of the launch when they share one
// (TM_SHARED: all stage a shared field; TM_GLOBAL: all add to their global
// field; TM_NONE: none keeps a field), else TM_AUTO (per instance): a launch
// whose instances agree runs without the code of the other modes.
template <typename R, int TM, bool GEN = false>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance_batch(Params<R> P) {
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ int sSeg;
    BatchSmem L;
    L.init<R>(P.bNt, P.bNw, P.bSdBytes, P.bTal);
    const InstD<R>* I = reinterpret_cast<const InstD<R>*>(smraw + L.inst);
    Window<R> W;
    W.init(P);
    blkZero();
    int cur = P.home[blockIdx.x];
    int curInst = -1;
    for (int bind = 0; bind < (1 << 30); ++bind) {
        if (threadIdx.x == 0) {
            int pick = -1;
            for (int k = 0; k < P.nseg; ++k) {
                int sg = cur + k;
                if (sg >= P.nseg) sg -= P.nseg;
                const SegD& G = P.segs[sg];
                const unsigned long long taken = *reinterpret_cast<volatile unsigned long long*>(P.segNext + sg);
                if (taken < (unsigned long long)(G.end - G.beg)) { pick = sg; break; }
            }
            sSeg = pick;
        }
        __syncthreads();
        const int sg = sSeg;
        if (sg < 0) break;
        cur = sg;
        const SegD S = P.segs[sg];
        if (S.inst != curInst) {
            stageInstance<R>(P, S.inst, smraw, L);
            curInst = S.inst;
        }
        __syncthreads();
        // a served instance may end its horizon in this window while others
        // are in the middle of theirs
        Window<R> Wb = W;
        Wb.last = W.last || (I->flags & IF_LAST) != 0;
        dynamicLoop<R, false, false, TM, BatchView<R>, GEN>(P, P.segNext + sg, (unsigned long long)S.beg,
                                              (unsigned long long)S.end, BatchView<R>{&P, smraw, I}, Wb);
        __syncthreads();
        flushBinding<R>(*I, S.group);
        __syncthreads();
    }
    flushCounts(P.counters);
}

// Shared memory of the batched kernel.
template <typename R>
__host__ __device__ inline size_t batchSmemBytes(const Params<R>& P) {
    BatchSmem L;
    L.init<R>(P.bNt, P.bNw, P.bSdBytes, P.bTal);
    return L.total;
}

// The batched layout's offsets into P (host, after the capacities).
template <typename R>
inline void setBatchLayout(Params<R>& P) {
    BatchSmem L;
    L.init<R>(P.bNt, P.bNw, P.bSdBytes, P.bTal);
    P.smVel = (int)L.vel;
    P.smVt = (int)L.vt;
    P.smWthr = (int)L.wthr;
    P.smGuide = (int)L.guide;
    P.smSd = (int)L.sd;
    P.smTal = (int)L.tal;
    P.smSplit = 0;
    P.smStage = 0;
}

// Global difference arrays -> field: block (i, y) prefix-sums row
// y % maxRows of field copy y / maxRows of instance i and adds it to that
// copy.
template <typename R>
__global__ void __launch_bounds__(32) k_difprefix(Params<R> P) {
    const InstD<R>& I = P.insts[blockIdx.x];
    const int r = (int)(blockIdx.y % (unsigned)P.maxRows), grp = (int)(blockIdx.y / (unsigned)P.maxRows);
    if (r >= I.rows || grp >= I.groups || I.gdif == nullptr) return;
    if (P.lastOnly && !(I.flags & IF_LAST)) return;
    const long long go = (long long)grp * I.gstride;
    const int lane = threadIdx.x;
    double carry = 0.0;
    const double* dr = I.gdif + go + (size_t)r * (I.cols + 1);
    for (int c0 = 0; c0 < I.cols; c0 += 32) {
        const int c = c0 + lane;
        double x = c < I.cols ? dr[c] : 0.0;
        for (int o = 1; o < 32; o <<= 1) {
            double y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        x += carry;
        if (c < I.cols) I.tally[go + (size_t)c * I.rows + r] += x;
        carry = __shfl_sync(0xFFFFFFFFu, x, 31);
    }
}

// End of a served round, block (x, i): gsum[i][g][r] = checksum of row r
// of field copy g (the batch-mean samples: the amount of every flight of the
// copy's phonons, equal to the copy's field summed over cells), and, for a
// solve that keeps its field, acc += the sum of its field copies. With
// lastOnly, instances whose round goes on are skipped.
constexpr int MAX_GROUPS = 8;

template <typename R>
__global__ void __launch_bounds__(256) k_round_reduce(Params<R> P, double* const* accs, double* gsum) {
    const InstD<R>& I = P.insts[blockIdx.y];
    if (P.lastOnly && !(I.flags & IF_LAST)) return;
    if (blockIdx.x == 0 && threadIdx.x < 4 * MAX_GROUPS) {
        const int g = threadIdx.x >> 2, r = threadIdx.x & 3;
        gsum[(long long)blockIdx.y * MAX_GROUPS * 4 + threadIdx.x] = (g < I.groups && r < I.rows) ? I.csum[threadIdx.x] : 0.0;
    }
    double* a = accs[blockIdx.y];
    if (a == nullptr || I.tally == nullptr) return;
    const int n = I.rows * I.cols;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int g = 0; g < I.groups; ++g) s += I.tally[(long long)g * I.gstride + e];
        a[e] += s;
    }
}

// Stream compaction of the live slots of a dynamic-kernel state into the
// other half (order of arrival per warp).
template <typename R>
__global__ void __launch_bounds__(256) k_compact(Params<R> P) {
    const unsigned long long n = P.live_in[0];
    const int lane = threadIdx.x & 31;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long i = base + threadIdx.x;
        uint4 A2 = make_uint4(0, PROP_DEAD, 0, 0);
        if (i < n) A2 = __ldcs(P.P2in + i);
        const bool live = !(A2.y & PROP_DEAD);
        const unsigned m = __ballot_sync(0xFFFFFFFFu, live);
        unsigned long long b = 0;
        if (lane == 0 && m) b = atomicAdd(&P.live_out[0], (unsigned long long)__popc(m));
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (live) {
            const unsigned long long o = b + __popc(m & ((1u << lane) - 1u));
            typename Vec4<R>::T A0, A1;
            ld4(P.P0in + i, A0);
            ld4(P.P1in + i, A1);
            st4(P.P0out + o, A0);
            st4(P.P1out + o, A1);
            __stcs(P.P2out + o, A2);
        }
    }
}

}  // namespace mcg
