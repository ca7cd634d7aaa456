// mc_device.cuh -- device building blocks of the phonon particle-advance
// kernels: parameters, random numbers, samplers, state packing.
//
// One thread owns one phonon. A launch advances every live phonon through a
// time window of K dt-steps, event by event (montecarlo/problem.cpp:401-435):
// nearest approaching face versus the free path (Subdomain::advect,
// montecarlo/subdomain.cpp:161-192), the flight tallied cell by cell
// (Field::accumulate, montecarlo/field.cpp:160-288), then the boundary event
// (montecarlo/boundary.cpp:283-287,308-312,349-359,455-460,516-522) or the
// relaxation-time scatter (montecarlo/material.cpp:287-303). Survivors are
// written, compacted by warp ballot + one atomic per warp, to the other half
// of a ping-pong structure of arrays.
//
// Positions are kept in the subdomain's reduced coordinates
// u = S * M^-1 (x - o) (S = max(div, 1)), split into an integer cell index
// and a Real offset inside the cell, so that flight arithmetic has cell-size
// rather than domain-size resolution; the subdomain faces are u_k = 0 and
// u_k = S_k and the tally cells are the unit cubes of u.
//
// Random numbers: Philox4x32-10 keyed by the seed with counter
// (phonon id, event index, block, 0); event 0 is the emission and event
// i + 1 the i-th loop iteration, so a phonon's draws do not depend on which
// thread, launch or ordering processed it. REPLAY mode reads a recorded
// per-phonon stream of 32-bit words instead.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mc_layout.h"

namespace mcg {

template <typename R> struct Vec4;
template <> struct Vec4<float> { using T = float4; };
struct __align__(32) dbl4 { double x, y, z, w; };
template <> struct Vec4<double> { using T = dbl4; };

// Limits of the two precisions.
template <typename R> struct Lim;
template <> struct Lim<float> {
    static __device__ __forceinline__ float tiny() { return 1.17549435e-38f; }
};
template <> struct Lim<double> {
    static __device__ __forceinline__ double tiny() { return 2.2250738585072014e-308; }
};

// ------------------------------------------------------------------ params
template <typename R> struct InstD;

// A work segment of a batched advance: the slots [beg, end) of one
// instance whose phonons all add to one field copy (batch-mean group).
struct SegD {
    long long beg, end;
    int inst, group;
};

// InstD::flags: a batched block stages the fixed-point field / the
// subdomain images in shared memory; the instance keeps no field (only the
// per-flight checksums, e.g. for kappa alone)
// IF_LAST: this launch's window is the last of the instance's horizon (a
// served round whose windows started at another launch than the others')
enum { IF_TAL_SHARED = 1, IF_SD_SHARED = 2, IF_NO_FIELD = 4, IF_LAST = 8 };

template <typename R>
struct Params {
    const SdomD<R>* sd;
    int nsd;
    const EmitterD* em;
    const long long* emitCdf;  // cumulative phonons per emitter
    int nem;
    // material tables
    int nw, np;
    const R* vel;   // nw x np
    const R* vt;    // vel * tau, nw x np
    const unsigned long long* wthr;   // scatter bin thresholds, nw
    const uint16_t* wguide;           // scatter bin guide table, GUIDE entries
    const unsigned long long* pthr;   // scatter branch thresholds, nw x np
    const unsigned long long* fwthr;  // flux (emission) bin thresholds
    const unsigned long long* fpthr;
    // problem
    int problem, rows, cols;
    int cumStep;  // CumTemp / CumFlux: scatters per bin, ceil((maxscat - 1) / size)
    long long nemit, maxscat, maxloop;
    R dt;
    int step0, ksteps, nsteps;
    // the window of this launch, derived from step0 on the host (setWindow)
    int wKeff, wLast;
    R wLen, wInvdt, wNext;
    // byte offsets in shared memory of the vel*tau table, scatter
    // thresholds, guide table, subdomain images and fixed-point field, and
    // of the static kernel's state stages: the single-instance layout
    // (setSingleLayout, vel at 0) or, in batched launches, the batched one
    // (setBatchLayout)
    int smVt, smWthr, smGuide, smSd, smTal, smStage;
    int smSplit;       // carry-free lean-flight field, 0 if none
    int tabGlobal;     // 1: vel * tau and the guide table read from global memory
    int smVel;  // batched launches: their layout's vel table (0 otherwise)
    uint32_t key0, key1;
    // state (ping-pong halves chosen by the host)
    typename Vec4<R>::T* P0in; typename Vec4<R>::T* P1in; uint4* P2in;
    typename Vec4<R>::T* P0out; typename Vec4<R>::T* P1out; uint4* P2out;
    // live phonons: the input holds [0, live_in[0]) and
    // [cap - live_in[1], cap); survivors whose next event falls inside the
    // next window are written from the front of the output, the others
    // from the back, so that warps see phonons of one kind
    const unsigned long long* live_in;
    unsigned long long* live_out;
    // single-instance dynamic launches of long windows: the launch-wide
    // slot counter every block claims from (zeroed before each launch);
    // null: each block claims from its own share of the slots
    unsigned long long* qglobal;
    unsigned long long cap;
    // static schedule: block b of the (fixed) grid owns the slots
    // [b regCap, (b + 1) regCap) of each half; its live phonons are the
    // regIn[2b] slots from the front of its region (next event inside
    // this window) and the regIn[2b + 1] slots at its back (no event in
    // it). Survivors go to the same region of the other half, counted in
    // regOut.
    unsigned int* regIn;
    unsigned int* regOut;
    long long regCap;
    // fixed-point quantum of the per-block shared tally and of the
    // per-thread checksums, per row
    R tqinv[4];
    double tq[4];
    unsigned long long* counters;
    unsigned int* status;
    double* tally;  // rows x cols, column-major
    double* csum;   // rows: sum over all flights of amount (tally checksum)
    // replay
    const uint32_t* rwords;
    const long long* roff;  // nemit + 1
    uint32_t* rcur;         // per phonon id
    // event log: logcap records x 12 doubles per phonon id < logn
    double* log;
    long long logcap, logn;
    int* logcount;
    // batched launches: instance descriptors and their slot offsets
    // (instance i owns slots [islot[i], islot[i+1]) of [0, cap))
    const InstD<R>* insts;
    const long long* islot;
    int ninst;
    int maxGroups;  // largest field-copy count of the instances
    int maxRows;    // largest row count of the instances
    // served windows: the round-end kernels (difference-array prefix, round
    // reduction) skip the instances without IF_LAST
    int lastOnly;
    // work segments of a batched advance: each block starts on segment
    // home[block] and moves on to any segment with slots left; segNext[s]
    // counts the slots of segment s already claimed
    const SegD* segs;
    const int* home;
    unsigned long long* segNext;
    int nseg;
    // shared-memory capacities of a batched block (largest instance that
    // stages its tables / subdomains / fixed-point field there)
    int bNt, bNw, bSdBytes, bTal;
};

// One problem instance as the advance loop sees it: material tables,
// domain, stop rules, field targets. A single-instance launch builds one in
// shared memory around its staged tables; a batched launch keeps one per
// instance in shared memory and each lane uses its phonon's.
template <typename R>
struct InstD {
    const R* vel;                     // nw x np
    const R* vt;                      // vel * tau
    const unsigned long long* wthr;   // scatter bin thresholds
    const uint16_t* wguide;           // scatter bin guide table
    const unsigned long long* pthr;   // scatter branch thresholds
    const unsigned long long* fwthr;  // flux (emission) thresholds
    const unsigned long long* fpthr;
    const SdomD<R>* sd;
    const EmitterD* em;
    const long long* emitCdf;         // cumulative phonons per emitter
    int nw, np, nem, nsd;
    int problem, rows, cols, inst;
    int cumStep;                      // CumTemp / CumFlux scatters per bin
    long long maxscat, maxloop;
    long long slot0, nemit;           // the instance's state slots
    uint32_t key0, key1;
    long long* tal;                   // shared fixed-point field (single instance)
    long long* dif;                   // its difference array
    double* tally;                    // global field, rows x cols column-major
    double* gdif;                     // global difference array, rows x (cols + 1), or null
    double* csum;                     // per-row checksums, 4 per field copy
    int groups;                       // phonon id % groups picks a field copy
    int flags;                        // IF_*: what a batched block stages
    long long gstride;                // doubles between field copies (tally and gdif)
    R tqinv[4];
    double tq[4];
};

// ------------------------------------------------------------------ RNG
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t& o0, uint32_t& o1,
                                              uint32_t& o2, uint32_t& o3) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    o0 = c0; o1 = c1; o2 = c2; o3 = c3;
}

// One Philox block out of line: the event code draws from several call
// sites, and one shared copy of the ten rounds keeps the advance loop small
// enough for the instruction cache.
static __device__ __noinline__ uint4 philoxBlock(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t k0, uint32_t k1) {
    uint4 o;
    philox4x32_10(c0, c1, c2, 0u, k0, k1, o.x, o.y, o.z, o.w);
    return o;
}

template <bool REPLAY> struct Rng;

template <> struct Rng<false> {
    uint32_t k0, k1, id, event, block, b0, b1, b2, b3;
    int lane;
    template <typename P>
    __device__ void init(uint32_t key0, uint32_t key1, uint32_t pid, const P*) {
        k0 = key0; k1 = key1; id = pid; event = 0; block = 0; lane = 0;
    }
    __device__ __forceinline__ void setEvent(uint32_t e) { event = e; block = 0; lane = 0; }
    // make the next block now if the current one is used up (next() then
    // finds words ready): lets the lanes that will draw make it together
    __device__ __forceinline__ void fill() {
        if (lane == 0) {
            const uint4 o = philoxBlock(id, event, block, k0, k1);
            b0 = o.x; b1 = o.y; b2 = o.z; b3 = o.w;
            ++block;
            lane = 4;
        }
    }
    __device__ __forceinline__ uint32_t next() {
        if (lane == 0) {
            const uint4 o = philoxBlock(id, event, block, k0, k1);
            b0 = o.x; b1 = o.y; b2 = o.z; b3 = o.w;
            ++block;
            lane = 4;
        }
        uint32_t x = b0;
        b0 = b1; b1 = b2; b2 = b3;
        --lane;
        return x;
    }
    __device__ __forceinline__ bool exhausted() const { return false; }
    __device__ __forceinline__ void save() {}
};

template <> struct Rng<true> {
    const uint32_t* w;
    long long pos, end;
    uint32_t* cur;
    long long start;
    bool ex;
    template <typename P>
    __device__ void init(uint32_t, uint32_t, uint32_t pid, const P* p) {
        start = p->roff[pid];
        end = p->roff[pid + 1];
        cur = p->rcur + pid;
        pos = start + *cur;
        w = p->rwords;
        ex = false;
    }
    __device__ __forceinline__ void setEvent(uint32_t) {}
    __device__ __forceinline__ void fill() {}
    __device__ __forceinline__ uint32_t next() {
        if (pos < end) return w[pos++];
        ex = true;
        return 0x80000000u;
    }
    __device__ __forceinline__ bool exhausted() const { return ex; }
    __device__ __forceinline__ void save() { *cur = (uint32_t)(pos - start); }
};

// Uniform conversions. FP64 follows boost's uniform_01 / uniform_real on a
// 32-bit engine exactly (u = x / 2^32); FP32 rounds the exact value once
// (u01 keeps the top 24 bits so that it stays below 1).
template <typename R> __device__ __forceinline__ R u01(uint32_t x);
template <> __device__ __forceinline__ double u01<double>(uint32_t x) { return (double)x * 0x1p-32; }
template <> __device__ __forceinline__ float u01<float>(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }
template <typename R> __device__ __forceinline__ R uone(uint32_t x);
template <> __device__ __forceinline__ double uone<double>(uint32_t x) { return (double)x * 0x1p-32 * 2.0 + (-1.0); }
template <> __device__ __forceinline__ float uone<float>(uint32_t x) {
    // 2u - 1 = (2x - 2^32) / 2^32, rounded once
    return __ll2float_rn(2LL * (long long)x - 0x100000000LL) * 0x1p-32f;
}
// -log(1 - u) with 1 - u formed exactly as (2^32 - x) / 2^32
__device__ __forceinline__ double neglog1m(uint32_t x, double) {
    return -log((double)(0x100000000ull - (unsigned long long)x) * 0x1p-32);
}
__device__ __forceinline__ float neglog1m(uint32_t x, float) {
    return -logf(__ull2float_rn(0x100000000ull - (unsigned long long)x) * 0x1p-32f);
}
__device__ __forceinline__ void sincospi_(double v, double* s, double* c) { sincospi(v, s, c); }
__device__ __forceinline__ void sincospi_(float v, float* s, float* c) { sincospif(v, s, c); }
__device__ __forceinline__ double sqrt_(double v) { return sqrt(v); }
__device__ __forceinline__ float sqrt_(float v) { return sqrtf(v); }

// Polar parts of the direction samplers from one 32-bit word x, u = x/2^32.
// FP64 follows the reference's arithmetic; FP32 forms 1 - c^2 = 4u(1-u) and
// |2u - 1|, 1 - |2u - 1| from exact integers so that the square roots do
// not amplify the 24-bit rounding of u near the poles.
__device__ __forceinline__ void isoPolar(uint32_t x, double& c, double& s) {
    c = uone<double>(x);
    s = sqrt(fmax(0.0, 1.0 - c * c));
}
__device__ __forceinline__ void isoPolar(uint32_t x, float& c, float& s) {
    const long long d2 = 2LL * (long long)x - 0x100000000LL;  // 2^32 (2u - 1)
    c = __ll2float_rn(d2) * 0x1p-32f;
    const float u = __uint2float_rn(x) * 0x1p-32f;
    const float v = __ull2float_rn(0x100000000ull - (unsigned long long)x) * 0x1p-32f;
    s = 2.0f * sqrtf(u * v);
}
__device__ __forceinline__ void anisoPolar(uint32_t x, bool bidir, double& c, double& s) {
    double r = uone<double>(x);
    double sg = (bidir && r < 0.0) ? -1.0 : 1.0;
    double s2 = fabs(r);
    s = sqrt(s2);
    c = sg * sqrt(1.0 - s2);
}
__device__ __forceinline__ void anisoPolar(uint32_t x, bool bidir, float& c, float& s) {
    const long long d2 = 2LL * (long long)x - 0x100000000LL;  // 2^32 r
    const bool neg = d2 < 0;
    const float sg = (bidir && neg) ? -1.0f : 1.0f;
    s = sqrtf(__ull2float_rn((unsigned long long)(neg ? -d2 : d2)) * 0x1p-32f);
    // 1 - |r| = 2 (1 - u) for r >= 0, 2 u for r < 0
    const unsigned long long q = neg ? 2ull * x : 2ull * (0x100000000ull - (unsigned long long)x);
    c = sg * sqrtf(__ull2float_rn(q) * 0x1p-32f);
}

// montecarlo/random.cpp:16-27
template <typename R, typename G>
__device__ __forceinline__ void drawIso(G& g, R d[3]) {
    R c, s;
    isoPolar(g.next(), c, s);
    R sp, cp;
    sincospi_(uone<R>(g.next()), &sp, &cp);
    d[0] = s * cp; d[1] = s * sp; d[2] = c;
}

// montecarlo/random.cpp:29-44
template <typename R, typename G>
__device__ __forceinline__ void drawAniso(G& g, bool bidir, R d[3]) {
    R c, s;
    anisoPolar(g.next(), bidir, c, s);
    R sp, cp;
    sincospi_(uone<R>(g.next()), &sp, &cp);
    d[0] = s * cp; d[1] = s * sp; d[2] = c;
}

template <typename R>
__device__ __forceinline__ void rotate(const R* m, const R v[3], R o[3]) {
    o[0] = (m[0] * v[0] + m[1] * v[1]) + m[2] * v[2];
    o[1] = (m[3] * v[0] + m[4] * v[1]) + m[5] * v[2];
    o[2] = (m[6] * v[0] + m[7] * v[1]) + m[8] * v[2];
}

// Phonon::dir normalisation (montecarlo/phonon.cpp:179-184)
__device__ __forceinline__ void normalize(double d[3]) {
    double z = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
    double s = sqrt(z);
    d[0] /= s; d[1] /= s; d[2] /= s;
}
__device__ __forceinline__ void normalize(float d[3]) {
    float z = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
    float s = rsqrtf(z);
    d[0] *= s; d[1] *= s; d[2] *= s;
}

// Inverse-CDF draw on integer thresholds: first i with x < thr[i]
// (equivalent to u < cdf[i] in FP64 for u = x / 2^32).
__device__ __forceinline__ int searchThr(const unsigned long long* thr, int n, uint32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((unsigned long long)x < thr[mid]) hi = mid; else lo = mid + 1;
    }
    return lo < n ? lo : n - 1;
}
// Guide-table search (Chen and Asau's indexed search): guide[k] is the
// answer for x = k * 2^32 / GUIDE, a lower bound for every x in slot k, so a
// short upward scan finishes the search.
constexpr int GUIDE_BITS = 10;
constexpr int GUIDE = 1 << GUIDE_BITS;
__device__ __forceinline__ int searchGuided(const unsigned long long* thr, const uint16_t* guide, int n, uint32_t x) {
    int i = guide[x >> (32 - GUIDE_BITS)];
    while (i < n - 1 && (unsigned long long)x >= thr[i]) ++i;
    return i;
}
__device__ __forceinline__ int searchBranch(const unsigned long long* thr, int np, uint32_t x) {
    for (int j = 0; j < np - 1; ++j)
        if ((unsigned long long)x < thr[j]) return j;
    return np - 1;
}

// ----------------------------------------------------------- state packing
__device__ __forceinline__ uint32_t packCell(int s, const int idx[3]) {
    return ((uint32_t)s << (3 * CELL_BITS)) | ((uint32_t)idx[0] << (2 * CELL_BITS)) |
           ((uint32_t)idx[1] << CELL_BITS) | (uint32_t)idx[2];
}
__device__ __forceinline__ void unpackCell(uint32_t c, int& s, int idx[3]) {
    const uint32_t m = (1u << CELL_BITS) - 1;
    s = (int)(c >> (3 * CELL_BITS));
    idx[0] = (int)((c >> (2 * CELL_BITS)) & m);
    idx[1] = (int)((c >> CELL_BITS) & m);
    idx[2] = (int)(c & m);
}
// prop word: w (16 bits) | p (8 bits) | negative sign (bit 24)
__device__ __forceinline__ uint32_t packProp(int w, int p, bool neg) {
    return (uint32_t)w | ((uint32_t)p << 16) | (neg ? (1u << 24) : 0u);
}

template <typename R>
__device__ __forceinline__ R idToReal(uint32_t id);
template <> __device__ __forceinline__ float idToReal<float>(uint32_t id) { return __uint_as_float(id); }
template <> __device__ __forceinline__ double idToReal<double>(uint32_t id) { return (double)id; }
template <typename R>
__device__ __forceinline__ uint32_t realToId(R v);
template <> __device__ __forceinline__ uint32_t realToId<float>(float v) { return __float_as_uint(v); }
template <> __device__ __forceinline__ uint32_t realToId<double>(double v) { return (uint32_t)v; }

__device__ __forceinline__ void ld4(const float4* p, float4& v) { v = __ldcs(p); }
__device__ __forceinline__ void ld4(const dbl4* p, dbl4& v) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldcs(q), b = __ldcs(q + 1);
    v.x = a.x; v.y = a.y; v.z = b.x; v.w = b.y;
}
__device__ __forceinline__ void st4(float4* p, const float4& v) { __stcs(p, v); }
__device__ __forceinline__ void st4(dbl4* p, const dbl4& v) {
    double2* q = reinterpret_cast<double2*>(p);
    __stcs(q, make_double2(v.x, v.y));
    __stcs(q + 1, make_double2(v.z, v.w));
}

}  // namespace mcg
