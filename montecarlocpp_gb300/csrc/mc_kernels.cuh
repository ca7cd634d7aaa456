// mc_kernels.cuh -- sm_103a kernels of the phonon particle-advance hot path.
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
    long long nemit, maxscat, maxloop;
    R dt;
    int step0, ksteps, nsteps;
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
    unsigned long long cap;
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

template <bool REPLAY> struct Rng;

template <> struct Rng<false> {
    uint32_t k0, k1, id, event, block, b0, b1, b2, b3;
    int lane;
    template <typename P>
    __device__ void init(uint32_t key0, uint32_t key1, uint32_t pid, const P*) {
        k0 = key0; k1 = key1; id = pid; event = 0; block = 0; lane = 0;
    }
    __device__ __forceinline__ void setEvent(uint32_t e) { event = e; block = 0; lane = 0; }
    __device__ __forceinline__ uint32_t next() {
        if (lane == 0) {
            philox4x32_10(id, event, block, 0u, k0, k1, b0, b1, b2, b3);
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

// ---------------------------------------------------------------- tables
template <typename R>
struct Smem {
    R* vel;
    R* vt;
    unsigned long long* wthr;
    uint16_t* wguide;
    const SdomD<R>* sd;  // subdomains (shared when they fit, else global)
    long long* tal;      // rows x cols fixed-point partial field (r * cols + c)
    long long* dif;      // rows x (cols + 1) difference array, fixed point
};

// Shared layout: vel and vel*tau tables, the scatter bin thresholds and
// guide table, the subdomains (when staged), then the block's tally.
struct SmemLayout {
    size_t vel, vt, wthr, guide, sd, tal, total;
    template <typename R>
    __host__ __device__ void init(int nw, int np, int nsdShared, int rows, int cols, bool sharedTally) {
        auto al = [](size_t b) { return (b + 15) & ~(size_t)15; };
        const size_t nt = (size_t)nw * np;
        vel = 0;
        vt = vel + sizeof(R) * nt;
        wthr = al(vt + sizeof(R) * nt);
        guide = al(wthr + sizeof(unsigned long long) * (size_t)nw);
        sd = al(guide + sizeof(uint16_t) * GUIDE);
        tal = al(sd + sizeof(SdomD<R>) * (size_t)nsdShared);
        total = tal + (sharedTally ? sizeof(long long) * (size_t)rows * (2 * (size_t)cols + 1) : 0);
    }
};

// Subdomain images staged in shared memory up to this many bytes.
constexpr size_t SD_SHARED_MAX = 32 * 1024;

__host__ __device__ inline size_t smemTallyBytes(int rows, int cols) {
    return sizeof(long long) * (size_t)rows * (2 * (size_t)cols + 1);
}

// Tally modes: per-block shared histogram (64-bit fixed point, exact and
// order-independent adds) flushed with FP64 atomics, or FP64 atomics
// straight to the global field (fields too large for shared memory).
enum { TM_SHARED = 0, TM_GLOBAL = 1 };

// Hard cap on events one thread processes in one launch (a guard: a
// phonon that reaches it is killed and flagged non-finite).
constexpr int MAX_EVENTS_PER_LAUNCH = 1 << 22;

// Resident blocks of 256 threads per SM the FP32 advance kernels are
// compiled for (register budget 65536 / (256 x this)).
#ifndef MC_MIN_BLOCKS_F32
#define MC_MIN_BLOCKS_F32 4
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

// Round a float to the nearest int64 with integer instructions only (the
// float -> int64 conversion runs on GB300's narrow FP64 pipe). |v| < 2^61.
__device__ __forceinline__ long long toFixed(float v) {
    const uint32_t b = __float_as_uint(v);
    const int e = (int)((b >> 23) & 0xFFu) - 150;  // v = m * 2^e
    const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u);
    long long r;
    if (e >= 0) r = m << e;
    else if (e > -25) r = (m + (1LL << (-e - 1))) >> (-e);
    else r = 0;
    return (b >> 31) ? -r : r;
}
__device__ __forceinline__ long long toFixed(double v) { return __double2ll_rn(v); }

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

template <typename R, int TM>
struct Tally {
    const Params<R>* P;
    const Smem<R>* sm;
    int rows;
    // amount per metre of flight, rows entries: Temp sign/v; Flux sign*d
    R rho[4];

    // fixed-point amount of row r for path length t
    __device__ __forceinline__ long long fixedOf(int r, R t) const { return toFixed(rho[r] * (t * P->tqinv[r])); }
    __device__ __forceinline__ void atomShared(int r, int col, long long v) const {
        atomicAdd(reinterpret_cast<unsigned long long*>(&sm->tal[r * P->cols + col]), (unsigned long long)v);
    }
    __device__ __forceinline__ void atomRange(int r, int c0, int c1, long long v) const {
        unsigned long long* d = reinterpret_cast<unsigned long long*>(sm->dif + r * (P->cols + 1));
        atomicAdd(d + c0, (unsigned long long)v);
        atomicAdd(d + c1, (unsigned long long)(-v));
    }
    __device__ __forceinline__ void addGlobal(int col, R t) const {
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < rows) atomicAdd(&P->tally[(size_t)col * rows + r], toDouble(rho[r] * t));
    }
};

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

// 1-D flight along axis K (the only axis with cells): closed form of
// montecarlo/field.cpp:187-223 -- partial first and last cells, full
// interior cells through the difference array. In the shared layout the
// flight's whole fixed-point amount V is computed once and the last cell
// takes the integer remainder, so the cells add up to V exactly.
template <typename R, int TM, int K>
__device__ __forceinline__ void fly1d(Phn<R>& ph, const SdomD<R>& S, const R a[3], const R ia[3], R s,
                                      Tally<R, TM>& T, long long csum[4]) {
    const int cb = S.colbeg;
    const int b = ph.idx[K];
    const int n = S.shape[K];
    // displacement in cell units relative to the current cell
    const R du = ph.off[K] + s * a[K];
    int e = b + (int)floor(du);
    e = min(max(e, 0), n - 1);
    const int stride = S.tstride[K];
    const R inva = fabs(ia[K]);
    const int lo = min(b, e), hi = max(b, e);
    const R tfirst = (e > b ? (R(1) - ph.off[K]) : ph.off[K]) * inva;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if (r >= T.rows) break;
        const long long V = T.fixedOf(r, s);
        csum[r] += V;
        if (TM == TM_SHARED) {
            if (e == b) {
                T.atomShared(r, cb + b * stride, V);
            } else {
                const long long F = T.fixedOf(r, tfirst);
                const long long I = T.fixedOf(r, inva);
                T.atomShared(r, cb + b * stride, F);
                T.atomShared(r, cb + e * stride, V - F - (long long)(hi - lo - 1) * I);
                if (stride == 1) { if (hi - lo > 1) T.atomRange(r, cb + lo + 1, cb + hi, I); }
                else for (int c = lo + 1; c < hi; ++c) T.atomShared(r, cb + c * stride, I);
            }
        }
    }
    if (TM == TM_GLOBAL) {
        if (e == b) {
            T.addGlobal(cb + b * stride, s);
        } else {
            const R tlast = s - tfirst - (R)(hi - lo - 1) * inva;
            T.addGlobal(cb + b * stride, tfirst);
            T.addGlobal(cb + e * stride, fmax(tlast, R(0)));
            for (int c = lo + 1; c < hi; ++c) T.addGlobal(cb + c * stride, inva);
        }
    }
    ph.idx[K] = e;
    ph.off[K] = clamp01(du - (R)(e - b));
#pragma unroll
    for (int j = 0; j < 3; ++j)
        if (j != K) moveAxis(ph, S, j, ph.off[j] + s * a[j]);
}

// Flight of path length s from the current cell, tallied cell by cell
// (Field::accumulate, montecarlo/field.cpp:160-288, as a cell walk); adds
// the flight's fixed-point amount to the thread's checksums.
template <typename R, int TM>
__device__ __forceinline__ void fly(Phn<R>& ph, const SdomD<R>& S, const R a[3], const R ia[3], R s,
                                   Tally<R, TM>& T, long long csum[4]) {
    const int acc = S.accum;
    const int cb = S.colbeg;
    if (acc < 0) {
        // a single field column (or none): move only
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (r >= T.rows) break;
            const long long V = T.fixedOf(r, s);
            csum[r] += V;
            if (acc == -1 && TM == TM_SHARED) T.atomShared(r, cb, V);
        }
        if (acc == -1 && TM == TM_GLOBAL) T.addGlobal(cb, s);
#pragma unroll
        for (int k = 0; k < 3; ++k) moveAxis(ph, S, k, ph.off[k] + s * a[k]);
        return;
    }
    if (acc == 0) { fly1d<R, TM, 0>(ph, S, a, ia, s, T, csum); return; }
    if (acc == 1) { fly1d<R, TM, 1>(ph, S, a, ia, s, T, csum); return; }
    if (acc == 2) { fly1d<R, TM, 2>(ph, S, a, ia, s, T, csum); return; }
    // 2-D / 3-D: walk the cells (Amanatides-Woo)
#pragma unroll
    for (int r = 0; r < 4; ++r)
        if (r < T.rows) csum[r] += T.fixedOf(r, s);
    R rem = s;
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
        if (TM == TM_SHARED) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (r < T.rows) T.atomShared(r, col, T.fixedOf(r, tmin));
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

// -------------------------------------------------------------- emission
// FieldProblem::solve emission part (montecarlo/problem.cpp:386-399) and
// Emitter::emit (montecarlo/boundary.cpp:378-385). Writes phonon n to slot n
// of the front half-range.
template <typename R, bool REPLAY>
__global__ void __launch_bounds__(256) k_emit(Params<R> P) {
    long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= P.nemit) return;
    // emitter = upper_bound(emitCdf, n)
    int lo = 0, hi = P.nem;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (P.emitCdf[mid] <= n) lo = mid + 1; else hi = mid;
    }
    const EmitterD E = P.em[lo];
    const SdomD<R>& S = P.sd[E.sdom];
    Rng<REPLAY> g;
    g.init(P.key0, P.key1, (uint32_t)n, &P);
    g.setEvent(0);
    Phn<R> ph;
    ph.s = E.sdom;
    ph.id = (uint32_t)n;
    ph.nscat = 0; ph.nloop = 0;
    {   // drawFluxProp (montecarlo/material.cpp:277-280)
        uint32_t x1 = g.next(), x2 = g.next();
        ph.w = searchThr(P.fwthr, P.nw, x1);
        ph.p = searchBranch(P.fpthr + (size_t)ph.w * P.np, P.np, x2);
    }
    R u[3];
    R dir[3];
    if (E.face >= 0) {
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
    ph.scatNext = drawScatNext<R>(g, P.vt[ph.w * P.np + ph.p]);
    if (REPLAY) {
        g.save();
        if (g.exhausted()) atomicOr(P.status, (unsigned)S_REPLAY_EXHAUSTED);
    }
    typename Vec4<R>::T a, b;
    a.x = ph.off[0]; a.y = ph.off[1]; a.z = ph.off[2]; a.w = ph.scatNext;
    b.x = ph.d[0]; b.y = ph.d[1]; b.z = ph.d[2]; b.w = idToReal<R>(ph.id);
    st4(P.P0out + n, a);
    st4(P.P1out + n, b);
    __stcs(P.P2out + n, make_uint4(packCell(ph.s, ph.idx), packProp(ph.w, ph.p, ph.neg), 0u, 0u));
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
        keff = min(P.ksteps, P.nsteps - P.step0);
        len = (R)keff * P.dt;
        invdt = R(1) / P.dt;
        last = (P.step0 + keff >= P.nsteps);
        next = (R)min(P.ksteps, max(P.nsteps - P.step0 - keff, 0)) * P.dt;
    }
};

// Per-thread counters, reduced once per launch.
struct Counts {
    uint32_t steps = 0, events = 0, scat = 0, esc = 0, hor = 0, maxs = 0, maxl = 0, abs = 0, bad = 0;
};

// Dead marker in the prop word of a slot written back in place.
constexpr uint32_t PROP_DEAD = 1u << 25;

// One phonon in flight: its state and the launch-local quantities derived
// from it. iterate() runs one loop iteration of montecarlo/problem.cpp:401-435
// (flight to the next event or to the end of the window, its tally, the
// event); finish() closes the phonon's window.
template <typename R, bool REPLAY, bool LOG, int TM>
struct Walker {
    Phn<R> ph;
    const SdomD<R>* S;
    R a[3], ia[3];
    R v, iv, sg;
    R budget;
    R tnext;       // time to the next event after the window end
    int nev;
    int stop;      // 0 alive, else the counter of the stop reason
    Rng<REPLAY> g;

    __device__ __forceinline__ void load(const Params<R>& P, const Smem<R>& sm, const Window<R>& W,
                                         const typename Vec4<R>::T& A0, const typename Vec4<R>::T& A1,
                                         const uint4& A2) {
        unpackCell(A2.x, ph.s, ph.idx);
        ph.off[0] = A0.x; ph.off[1] = A0.y; ph.off[2] = A0.z; ph.scatNext = A0.w;
        ph.d[0] = A1.x; ph.d[1] = A1.y; ph.d[2] = A1.z;
        ph.id = realToId<R>(A1.w);
        ph.w = (int)(A2.y & 0xFFFFu);
        ph.p = (int)((A2.y >> 16) & 0xFFu);
        ph.neg = (A2.y >> 24) & 1u;
        ph.nscat = A2.z;
        ph.nloop = A2.w;
        g.init(P.key0, P.key1, ph.id, &P);
        budget = W.len;
        S = &sm.sd[ph.s];
        reducedVel(*S, ph.d, a, ia);
        v = sm.vel[ph.w * P.np + ph.p];
        iv = R(1) / v;
        sg = ph.neg ? R(-1) : R(1);
        stop = 0;
        nev = 0;
        tnext = R(0);
    }

    __device__ __forceinline__ void pack(typename Vec4<R>::T& A0, typename Vec4<R>::T& A1, uint4& A2) const {
        A0.x = ph.off[0]; A0.y = ph.off[1]; A0.z = ph.off[2]; A0.w = ph.scatNext;
        A1.x = ph.d[0]; A1.y = ph.d[1]; A1.z = ph.d[2]; A1.w = idToReal<R>(ph.id);
        A2.x = packCell(ph.s, ph.idx);
        A2.y = packProp(ph.w, ph.p, ph.neg);
        A2.z = ph.nscat;
        A2.w = ph.nloop;
    }

    // returns true when the phonon's window is over (alive or stopped)
    __device__ __forceinline__ bool iterate(const Params<R>& P, const Smem<R>& sm, const Window<R>& W,
                                            Tally<R, TM>& T, Counts& C, long long csum[4]) {
        // Subdomain::advect (montecarlo/subdomain.cpp:161-192): the
        // approaching face of each axis, in the reference's face order
        // (lower faces 0..2, then upper faces 3..5), against the free path;
        // strict < keeps the first of equals
        R sev = ph.scatNext;
        int face = -1;
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
        const R tev = sev * iv;
        const bool event = tev <= budget;
        const R s = event ? sev : budget * v;
        // tally amounts per metre (montecarlo/problem.cpp:473-544)
        if (P.problem == P_TEMP) { T.rho[0] = sg * iv; }
        else if (P.problem == P_FLUX) { T.rho[0] = sg * ph.d[0]; T.rho[1] = sg * ph.d[1]; T.rho[2] = sg * ph.d[2]; }
        else { T.rho[0] = sg * iv; T.rho[1] = sg * ph.d[0]; T.rho[2] = sg * ph.d[1]; T.rho[3] = sg * ph.d[2]; }
        const int sBefore = ph.s;
        int cellEnd = 0;
        fly<R, TM>(ph, *S, a, ia, s, T, csum);
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
        g.setEvent(ph.nloop + 1);
        if (face >= 0) {
            const FaceD<R>& F = S->f[face];
            // the flight ends on the face: snap that coordinate
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (face == k) { ph.idx[k] = 0; ph.off[k] = R(0); }
                if (face == k + 3) { ph.idx[k] = S->shape[k] - 1; ph.off[k] = R(1); }
            }
            switch (F.kind) {
            case F_SPEC: {  // montecarlo/boundary.cpp:283-287
                R nd = (F.n[0] * ph.d[0] + F.n[1] * ph.d[1]) + F.n[2] * ph.d[2];
                for (int j = 0; j < 3; ++j) ph.d[j] -= R(2) * nd * F.n[j];
                normalize(ph.d);
                break;
            }
            case F_DIFF: {  // montecarlo/boundary.cpp:308-312
                R vv[3];
                drawAniso<R>(g, false, vv);
                rotate(F.rot, vv, ph.d);
                normalize(ph.d);
                ph.nscat++;
                break;
            }
            case F_ISOT:  // montecarlo/boundary.cpp:455-460
                stop = C_ABSORBED;
                break;
            case F_PERI:     // montecarlo/boundary.cpp:516-522
            case F_INTER: {  // montecarlo/boundary.cpp:349-359 (single pair)
                if (F.to < 0) { stop = C_ESCAPES; break; }
                if (F.tang) {
                    // same axis, tangential cells unchanged: keep the split
                    // coordinates, move onto the paired face
                    ph.s = F.to;
                    S = &sm.sd[ph.s];
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        if (F.toface == j) { ph.idx[j] = 0; ph.off[j] = R(0); }
                        if (F.toface == j + 3) { ph.idx[j] = S->shape[j] - 1; ph.off[j] = R(1); }
                    }
                } else {
                    R u[3], u2[3];
                    for (int j = 0; j < 3; ++j) u[j] = (R)ph.idx[j] + ph.off[j];
                    rotate(F.A, u, u2);
                    for (int j = 0; j < 3; ++j) u2[j] += F.b[j];
                    ph.s = F.to;
                    S = &sm.sd[ph.s];
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        if (F.toface == j) u2[j] = R(0);
                        if (F.toface == j + 3) u2[j] = S->S[j];
                    }
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        int ii = (int)floor(u2[j]);
                        ii = min(max(ii, 0), S->shape[j] - 1);
                        ph.idx[j] = ii;
                        ph.off[j] = clamp01(u2[j] - (R)ii);
                    }
                }
                if (F.kind == F_PERI && !F.ident) {
                    R dd[3] = {ph.d[0], ph.d[1], ph.d[2]};
                    rotate(F.Rd, dd, ph.d);
                    normalize(ph.d);
                }
                break;
            }
            }
        } else {
            // Material::scatter (montecarlo/material.cpp:298-303)
            uint32_t x1 = g.next(), x2 = g.next();
            ph.w = searchGuided(sm.wthr, sm.wguide, P.nw, x1);
            ph.p = searchBranch(P.pthr + ph.w * P.np, P.np, x2);
            drawIso<R>(g, ph.d);
            normalize(ph.d);
            ph.nscat++;
            ph.scatNext = drawScatNext<R>(g, sm.vt[ph.w * P.np + ph.p]);
            v = sm.vel[ph.w * P.np + ph.p];
            iv = R(1) / v;
            ++C.scat;
        }
        ++C.events;
        if (LOG) logEvent(P, ph, sBefore, face, ph.s, xe, (double)P.step0 * (double)P.dt + (double)(W.len - budget),
                          cellEnd);
        ph.nloop++;
        if (REPLAY && g.exhausted()) { stop = C_REPLAY_EXHAUSTED; return true; }
        if (stop) return true;
        if ((long long)ph.nscat >= P.maxscat) { stop = C_MAXSCAT; return true; }
        if ((long long)ph.nloop >= P.maxloop) { stop = C_MAXLOOP; return true; }
        if (++nev >= MAX_EVENTS_PER_LAUNCH) { stop = C_BAD; return true; }
        reducedVel(*S, ph.d, a, ia);
        return false;
    }

    // the phonon's window is over: count its steps and its stop reason;
    // returns true if it stays alive
    __device__ __forceinline__ bool finish(const Params<R>& P, const Window<R>& W, Counts& C) {
        if (REPLAY) g.save();
        if (stop == 0) {
            C.steps += W.keff;
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
            int st = (int)ceil(el * W.invdt);
            st = st < 1 ? 1 : (st > W.keff ? W.keff : st);
            C.steps += st;
        }
        switch (stop) {
        case 0: break;
        case C_ESCAPES: ++C.esc; break;
        case C_HORIZON: ++C.hor; break;
        case C_MAXSCAT: ++C.maxs; break;
        case C_MAXLOOP: ++C.maxl; break;
        case C_ABSORBED: ++C.abs; break;
        case C_REPLAY_EXHAUSTED: atomicOr(P.status, (unsigned)S_REPLAY_EXHAUSTED); break;
        default: ++C.bad; atomicOr(P.status, (unsigned)S_NONFINITE); break;
        }
        return stop == 0;
    }
};

// Stage the material tables, the subdomains and (zeroed) the block's tally
// in shared memory.
template <typename R, int TM>
__device__ __forceinline__ void stageTables(const Params<R>& P, Smem<R>& sm, unsigned char* smraw) {
    const int nt = P.nw * P.np;
    const int nsdShared = (size_t)P.nsd * sizeof(SdomD<R>) <= SD_SHARED_MAX ? P.nsd : 0;
    SmemLayout L;
    L.init<R>(P.nw, P.np, nsdShared, P.rows, P.cols, TM == TM_SHARED);
    sm.vel = reinterpret_cast<R*>(smraw + L.vel);
    sm.vt = reinterpret_cast<R*>(smraw + L.vt);
    sm.wthr = reinterpret_cast<unsigned long long*>(smraw + L.wthr);
    sm.wguide = reinterpret_cast<uint16_t*>(smraw + L.guide);
    sm.tal = reinterpret_cast<long long*>(smraw + L.tal);
    sm.dif = sm.tal + (size_t)P.rows * P.cols;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        sm.vel[i] = P.vel[i];
        sm.vt[i] = P.vt[i];
    }
    for (int i = threadIdx.x; i < P.nw; i += blockDim.x) sm.wthr[i] = P.wthr[i];
    for (int i = threadIdx.x; i < GUIDE; i += blockDim.x) sm.wguide[i] = P.wguide[i];
    if (nsdShared) {
        const int nw4 = (int)(sizeof(SdomD<R>) * nsdShared / 4);
        uint32_t* dst = reinterpret_cast<uint32_t*>(smraw + L.sd);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(P.sd);
        for (int i = threadIdx.x; i < nw4; i += blockDim.x) dst[i] = src[i];
        sm.sd = reinterpret_cast<const SdomD<R>*>(smraw + L.sd);
    } else {
        sm.sd = P.sd;
    }
    if (TM == TM_SHARED) {
        const int nz = P.rows * (2 * P.cols + 1);
        for (int i = threadIdx.x; i < nz; i += blockDim.x) sm.tal[i] = 0;
    }
}

// Reduce the counters and checksums (one atomic per warp), then turn the
// block's difference array into cell values and flush the fixed-point field
// as FP64 atomics.
template <typename R, int TM>
__device__ __forceinline__ void closeBlock(const Params<R>& P, const Smem<R>& sm, const Counts& C,
                                           const long long csum[4]) {
    const int lane = threadIdx.x & 31;
    const uint32_t cs[9] = {C.steps, C.events, C.scat, C.esc, C.hor, C.maxs, C.maxl, C.abs, C.bad};
    const int ids[9] = {C_PHONON_STEPS, C_EVENTS, C_SCATTERS, C_ESCAPES, C_HORIZON, C_MAXSCAT,
                        C_MAXLOOP, C_ABSORBED, C_BAD};
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        unsigned long long x = cs[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if (lane == 0 && x) atomicAdd(&P.counters[ids[q]], x);
    }
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
            const long long* dr = sm.dif + r * (P.cols + 1);
            for (int c0 = 0; c0 < P.cols; c0 += 32) {
                const int c = c0 + lane;
                long long x = c < P.cols ? dr[c] : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (lane >= o) x += y;
                }
                x += carry;
                if (c < P.cols) sm.tal[r * P.cols + c] += x;
                carry = __shfl_sync(0xFFFFFFFFu, x, 31);
            }
        }
        __syncthreads();
        const int tot = P.rows * P.cols;
        for (int q = threadIdx.x; q < tot; q += blockDim.x) {
            const long long x = sm.tal[q];
            if (x != 0) {
                const int r = q / P.cols, c = q - r * P.cols;
                atomicAdd(&P.tally[(size_t)c * P.rows + r], (double)x * P.tq[r]);
            }
        }
    }
}

// Static kernel: one phonon per thread per pass of a grid-stride loop;
// survivors are compacted to the two ends of the other half of the
// ping-pong state (front: next event inside the next window).
template <typename R, bool REPLAY, bool LOG, int TM>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance(Params<R> P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    Smem<R> sm;
    stageTables<R, TM>(P, sm, smraw);
    __syncthreads();

    const unsigned long long nf = P.live_in[0], nb = P.live_in[1];
    const unsigned long long n = nf + nb;
    Window<R> W;
    W.init(P);
    long long csum[4] = {0, 0, 0, 0};
    Counts C;
    const int lane = threadIdx.x & 31;
    Tally<R, TM> T;
    T.P = &P;
    T.sm = &sm;
    T.rows = P.rows;
    T.rho[1] = T.rho[2] = T.rho[3] = R(0);

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
            wk.load(P, sm, W, A0, A1, A2);
            while (!wk.iterate(P, sm, W, T, C, csum)) {}
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
    closeBlock<R, TM>(P, sm, C, csum);
}

// Dynamic kernel: block b owns input slots [b C, (b + 1) C); each warp keeps
// its lanes busy by refilling finished lanes from the block's queue whenever
// at least REFILL of them are idle, so a long phonon no longer holds up its
// warp. Survivors are written back in place; dead slots get PROP_DEAD and are
// skipped until the host compacts. Input == output state half.
constexpr int REFILL = 8;

template <typename R, bool REPLAY, bool LOG, int TM>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? MC_MIN_BLOCKS_F32 : 2) k_advance_dyn(Params<R> P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ unsigned long long qnext;
    Smem<R> sm;
    stageTables<R, TM>(P, sm, smraw);
    const unsigned long long n = P.live_in[0];  // slots [0, n)
    const unsigned long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const unsigned long long qbeg = min((unsigned long long)blockIdx.x * chunk, n);
    const unsigned long long qend = min(qbeg + chunk, n);
    if (threadIdx.x == 0) qnext = qbeg;
    __syncthreads();

    Window<R> W;
    W.init(P);
    long long csum[4] = {0, 0, 0, 0};
    Counts C;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    Tally<R, TM> T;
    T.P = &P;
    T.sm = &sm;
    T.rows = P.rows;
    T.rho[1] = T.rho[2] = T.rho[3] = R(0);

    Walker<R, REPLAY, LOG, TM> wk;
    bool have = false;
    unsigned long long slot = 0;
    bool drained = false;
    uint32_t alive = 0;
    for (int guard = 0; guard < (1 << 30); ++guard) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !have);
        if (!drained && (idle == 0xFFFFFFFFu || __popc(idle) >= REFILL)) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&qnext, (unsigned long long)__popc(idle));
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
                        wk.load(P, sm, W, A0, A1, A2);
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
        if (have && wk.iterate(P, sm, W, T, C, csum)) {
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
    {
        unsigned long long x = alive;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if (lane == 0 && x) atomicAdd(&P.live_out[0], x);
    }
    closeBlock<R, TM>(P, sm, C, csum);
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
