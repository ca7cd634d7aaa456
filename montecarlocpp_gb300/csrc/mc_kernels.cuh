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
//   k_advance               static: one phonon per thread per pass; survivors
//                           compacted by warp ballot to the two ends of the
//                           other half of the state
//   k_advance_dyn           dynamic: warps refill idle lanes from a
//                           block-owned queue; state written back in place
//   k_advance_batch         dynamic, over many instances in one launch
//   k_compact               stream compaction of dead slots
//   k_difprefix             global difference arrays -> field (batched)
#pragma once

#include "mc_walker.cuh"

namespace mcg {

// Instance descriptor of a single-instance launch, around the tables it
// staged in shared memory.
template <typename R, int TM>
__device__ __forceinline__ InstD<R>* stageTables(const Params<R>& P, unsigned char* smraw) {
    const int nt = P.nw * P.np;
    const int nsdShared = (size_t)P.nsd * sizeof(SdomD<R>) <= SD_SHARED_MAX ? P.nsd : 0;
    SmemLayout L;
    L.init<R>(P.nw, P.np, nsdShared, P.rows, P.cols, TM == TM_SHARED);
    R* vel = reinterpret_cast<R*>(smraw + L.vel);
    R* vt = reinterpret_cast<R*>(smraw + L.vt);
    unsigned long long* wthr = reinterpret_cast<unsigned long long*>(smraw + L.wthr);
    uint16_t* wguide = reinterpret_cast<uint16_t*>(smraw + L.guide);
    long long* tal = reinterpret_cast<long long*>(smraw + L.tal);
    InstD<R>* I = reinterpret_cast<InstD<R>*>(smraw + L.inst);
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        vel[i] = P.vel[i];
        vt[i] = P.vt[i];
    }
    for (int i = threadIdx.x; i < P.nw; i += blockDim.x) wthr[i] = P.wthr[i];
    for (int i = threadIdx.x; i < GUIDE; i += blockDim.x) wguide[i] = P.wguide[i];
    const SdomD<R>* sd = P.sd;
    if (nsdShared) {
        const int nw4 = (int)(sizeof(SdomD<R>) * nsdShared / 4);
        uint32_t* dst = reinterpret_cast<uint32_t*>(smraw + L.sd);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(P.sd);
        for (int i = threadIdx.x; i < nw4; i += blockDim.x) dst[i] = src[i];
        sd = reinterpret_cast<const SdomD<R>*>(smraw + L.sd);
    }
    if (TM == TM_SHARED) {
        const int nz = P.rows * (2 * P.cols + 1);
        for (int i = threadIdx.x; i < nz; i += blockDim.x) tal[i] = 0;
    }
    if (threadIdx.x == 0) {
        I->vel = vel; I->vt = vt; I->wthr = wthr; I->wguide = wguide; I->pthr = P.pthr;
        I->fwthr = P.fwthr; I->fpthr = P.fpthr;
        I->sd = sd; I->em = P.em; I->emitCdf = P.emitCdf;
        I->nw = P.nw; I->np = P.np; I->nem = P.nem; I->nsd = P.nsd;
        I->problem = P.problem; I->rows = P.rows; I->cols = P.cols; I->inst = 0;
        I->maxscat = P.maxscat; I->maxloop = P.maxloop;
        I->slot0 = 0; I->nemit = P.nemit;
        I->key0 = P.key0; I->key1 = P.key1;
        I->tal = TM == TM_SHARED ? tal : nullptr;
        I->dif = TM == TM_SHARED ? tal + (size_t)P.rows * P.cols : nullptr;
        I->tally = P.tally; I->gdif = nullptr; I->csum = P.csum;
        I->groups = 1; I->gstride = 0;
        for (int r = 0; r < 4; ++r) { I->tqinv[r] = P.tqinv[r]; I->tq[r] = P.tq[r]; }
    }
    return I;
}

// End of a single-instance launch: counters and checksums (one atomic per
// warp), then the block's difference array turned into cell values and the
// fixed-point field flushed as FP64 atomics.
template <typename R, int TM>
__device__ __forceinline__ void closeBlock(const Params<R>& P, const InstD<R>& I, const Counts& C,
                                           const long long csum[4]) {
    const int lane = threadIdx.x & 31;
    flushCounts(P.counters, C);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        long long x = csum[r];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if (lane == 0 && r < P.rows && x != 0) atomicAdd(&P.csum[r], (double)x * P.tq[r]);
    }
    if (TM == TM_SHARED) {
        __syncthreads();
        const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        for (int r = warp; r < P.rows; r += nwarps) {
            long long carry = 0;
            const long long* dr = I.dif + r * (P.cols + 1);
            for (int c0 = 0; c0 < P.cols; c0 += 32) {
                const int c = c0 + lane;
                long long x = c < P.cols ? dr[c] : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (lane >= o) x += y;
                }
                x += carry;
                if (c < P.cols) I.tal[r * P.cols + c] += x;
                carry = __shfl_sync(0xFFFFFFFFu, x, 31);
            }
        }
        __syncthreads();
        const int tot = P.rows * P.cols;
        for (int q = threadIdx.x; q < tot; q += blockDim.x) {
            const long long x = I.tal[q];
            if (x != 0) {
                const int r = q / P.cols, c = q - r * P.cols;
                atomicAdd(&P.tally[(size_t)c * P.rows + r], (double)x * P.tq[r]);
            }
        }
    }
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

// Emission of every instance of a batch: slot n belongs to the instance whose
// slot range holds it; its phonon id is n - slot0.
template <typename R>
__global__ void __launch_bounds__(256) k_emit_batch(Params<R> P) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= (long long)P.cap) return;
    const InstD<R>& I = P.insts[instanceOf(P.islot, P.ninst, n)];
    const long long id = n - I.slot0;
    Rng<false> g;
    g.init(I.key0, I.key1, (uint32_t)id, &P);
    Phn<R> ph;
    emitOne<R>(I, id, g, ph);
    typename Vec4<R>::T a, b;
    uint4 c;
    packPhonon(ph, a, b, c);
    st4(P.P0out + n, a);
    st4(P.P1out + n, b);
    __stcs(P.P2out + n, c);
}

// ----------------------------------------------------------------- advance
// Static kernel: one phonon per thread per pass of a grid-stride loop;
// survivors are compacted to the two ends of the other half of the
// ping-pong state (front: next event inside the next window).
template <typename R, bool REPLAY, bool LOG, int TM>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance(Params<R> P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    InstD<R>* I = stageTables<R, TM>(P, smraw);
    __syncthreads();

    const unsigned long long nf = P.live_in[0], nb = P.live_in[1];
    const unsigned long long n = nf + nb;
    Window<R> W;
    W.init(P);
    long long csum[4] = {0, 0, 0, 0};
    Counts C;
    const int lane = threadIdx.x & 31;

    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long i = base + threadIdx.x;
        bool alive = false, soon = false;
        typename Vec4<R>::T A0, A1;
        uint4 A2;
        if (i < n) {
            const unsigned long long slot = i < nf ? i : P.cap - nb + (i - nf);
            ld4(P.P0in + slot, A0);
            ld4(P.P1in + slot, A1);
            A2 = __ldcs(P.P2in + slot);
            Walker<R, REPLAY, LOG, TM> wk;
            wk.load(P, I, W, A0, A1, A2);
            while (!wk.iterate(P, W, C, csum)) {}
            alive = wk.finish(P, W, C);
            soon = wk.tnext < W.next;
            if (alive) wk.pack(A0, A1, A2);
        }
        // fused compaction into two ends: one atomic per warp and end
        const unsigned mf = __ballot_sync(0xFFFFFFFFu, alive && soon);
        const unsigned mb = __ballot_sync(0xFFFFFFFFu, alive && !soon);
        unsigned long long bf = 0, bb = 0;
        if (lane == 0) {
            if (mf) bf = atomicAdd(&P.live_out[0], (unsigned long long)__popc(mf));
            if (mb) bb = atomicAdd(&P.live_out[1], (unsigned long long)__popc(mb));
        }
        bf = __shfl_sync(0xFFFFFFFFu, bf, 0);
        bb = __shfl_sync(0xFFFFFFFFu, bb, 0);
        if (alive) {
            const unsigned lt = (1u << lane) - 1u;
            const unsigned long long o = soon ? bf + __popc(mf & lt) : P.cap - 1 - (bb + __popc(mb & lt));
            st4(P.P0out + o, A0);
            st4(P.P1out + o, A1);
            __stcs(P.P2out + o, A2);
        }
    }
    closeBlock<R, TM>(P, *I, C, csum);
}

// Dynamic schedule shared by the single-instance and batched kernels: block
// b owns slots [b C, (b + 1) C) of [0, n); each warp keeps its lanes busy by
// refilling finished lanes from the block's queue whenever at least REFILL
// of them are idle, so a long phonon no longer holds up its warp. Survivors
// are written back in place; dead slots get PROP_DEAD (skipped until the
// host compacts). `inst(slot)` gives a slot's instance descriptor; BATCH
// flushes each phonon's checksum to its instance when its window ends.
constexpr int REFILL = 8;

template <typename R, bool REPLAY, bool LOG, int TM, bool BATCH, typename InstOf>
__device__ __forceinline__ void dynamicLoop(const Params<R>& P, unsigned long long n, unsigned long long* qnext,
                                            InstOf inst, const Window<R>& W, Counts& C, long long csum[4]) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const unsigned long long qbeg = min((unsigned long long)blockIdx.x * chunk, n);
    const unsigned long long qend = min(qbeg + chunk, n);
    Walker<R, REPLAY, LOG, TM> wk;
    bool have = false;
    unsigned long long slot = 0;
    bool drained = qbeg >= qend;
    uint32_t alive = 0;
    for (int guard = 0; guard < (1 << 30); ++guard) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !have);
        if (!drained && (idle == 0xFFFFFFFFu || __popc(idle) >= REFILL)) {
            unsigned long long b = 0;
            if (lane == 0) b = qbeg + atomicAdd(qnext, (unsigned long long)__popc(idle));
            b = __shfl_sync(0xFFFFFFFFu, b, 0);
            if (b + __popc(idle) >= qend) drained = true;
            if (!have) {
                const unsigned long long my = b + __popc(idle & lt);
                if (my < qend) {
                    typename Vec4<R>::T A0, A1;
                    uint4 A2 = __ldcs(P.P2in + my);
                    if (!(A2.y & PROP_DEAD)) {
                        ld4(P.P0in + my, A0);
                        ld4(P.P1in + my, A1);
                        wk.load(P, inst(my), W, A0, A1, A2);
                        have = true;
                        slot = my;
                        if (BATCH) csum[0] = csum[1] = csum[2] = csum[3] = 0;
                    }
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, have) == 0) {
            if (drained) break;
            continue;
        }
        if (have && wk.iterate(P, W, C, csum)) {
            if (BATCH) {
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (r < wk.I->rows && csum[r]) atomicAdd(&wk.I->csum[r], (double)csum[r] * wk.I->tq[r]);
            }
            typename Vec4<R>::T A0, A1;
            uint4 A2;
            if (wk.finish(P, W, C)) {
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

template <typename R>
struct SingleInst {
    const InstD<R>* I;
    __device__ __forceinline__ const InstD<R>* operator()(unsigned long long) const { return I; }
};

template <typename R>
struct BatchInst {
    const InstD<R>* sI;
    const long long* sSlot;
    int ninst;
    __device__ __forceinline__ const InstD<R>* operator()(unsigned long long slot) const {
        return &sI[instanceOf(sSlot, ninst, (long long)slot)];
    }
};

template <typename R, bool REPLAY, bool LOG, int TM>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance_dyn(Params<R> P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ unsigned long long qnext;
    InstD<R>* I = stageTables<R, TM>(P, smraw);
    if (threadIdx.x == 0) qnext = 0;
    __syncthreads();
    Window<R> W;
    W.init(P);
    long long csum[4] = {0, 0, 0, 0};
    Counts C;
    dynamicLoop<R, REPLAY, LOG, TM, false>(P, P.live_in[0], &qnext, SingleInst<R>{I}, W, C, csum);
    closeBlock<R, TM>(P, *I, C, csum);
}

// Batched kernel: the dynamic schedule over the slots of many instances at
// once (slots [islot[i], islot[i+1]) belong to instance i). Each lane runs
// its phonon against its instance's tables, domain and field. Fields are
// FP64 global atomics with global difference arrays (k_difprefix finishes
// them).
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance_batch(Params<R> P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ unsigned long long qnext;
    InstD<R>* sI = reinterpret_cast<InstD<R>*>(smraw);
    long long* sSlot = reinterpret_cast<long long*>(smraw + sizeof(InstD<R>) * P.ninst);
    {
        const int nw4 = (int)(sizeof(InstD<R>) * P.ninst / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(P.insts);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sI);
        for (int i = threadIdx.x; i < nw4; i += blockDim.x) dst[i] = src[i];
        for (int i = threadIdx.x; i <= P.ninst; i += blockDim.x) sSlot[i] = P.islot[i];
    }
    if (threadIdx.x == 0) qnext = 0;
    __syncthreads();
    Window<R> W;
    W.init(P);
    long long csum[4] = {0, 0, 0, 0};
    Counts C;
    dynamicLoop<R, false, false, TM_GLOBAL, true>(P, P.cap, &qnext, BatchInst<R>{sI, sSlot, P.ninst}, W, C, csum);
    flushCounts(P.counters, C);
}

// Shared memory of the batched kernel.
template <typename R>
__host__ __device__ inline size_t batchSmemBytes(int ninst) {
    return sizeof(InstD<R>) * (size_t)ninst + sizeof(long long) * ((size_t)ninst + 1);
}

// Global difference arrays -> field: block (i, y) prefix-sums row y % 4 of
// field copy y / 4 of instance i and adds it to that copy.
template <typename R>
__global__ void __launch_bounds__(32) k_difprefix(Params<R> P) {
    const InstD<R>& I = P.insts[blockIdx.x];
    const int r = blockIdx.y & 3, grp = blockIdx.y >> 2;
    if (r >= I.rows || grp >= I.groups || I.gdif == nullptr) return;
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

// End of a served round, block (x, i): over instance i's field copies,
// acc += sum of the copies, and gsum[i][g][r] = sum over cells of row r of
// copy g (the batch-mean samples), one atomic per warp and (g, r).
constexpr int MAX_GROUPS = 8;

template <typename R>
__global__ void __launch_bounds__(256) k_round_reduce(Params<R> P, double* const* accs, double* gsum) {
    const InstD<R>& I = P.insts[blockIdx.y];
    const int n = I.rows * I.cols;
    const int G = I.groups;
    double part[MAX_GROUPS][4];
#pragma unroll
    for (int g = 0; g < MAX_GROUPS; ++g)
#pragma unroll
        for (int r = 0; r < 4; ++r) part[g][r] = 0.0;
    double* a = accs[blockIdx.y];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int r = e % I.rows;
        double s = 0.0;
#pragma unroll
        for (int g = 0; g < MAX_GROUPS; ++g) {
            if (g < G) {
                const double v = I.tally[(long long)g * I.gstride + e];
                s += v;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q == r) part[g][q] += v;
            }
        }
        a[e] += s;
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int g = 0; g < MAX_GROUPS; ++g)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            double x = part[g][r];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
            if (lane == 0 && g < G && r < I.rows && x != 0.0) atomicAdd(&gsum[((long long)blockIdx.y * MAX_GROUPS + g) * 4 + r], x);
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
