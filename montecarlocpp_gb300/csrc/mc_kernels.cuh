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
    const unsigned long long* nlive_in;
    unsigned long long* nlive_out;
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
// 32-bit engine exactly (u = x / 2^32); FP32 keeps the top 24 bits.
template <typename R> __device__ __forceinline__ R u01(uint32_t x);
template <> __device__ __forceinline__ double u01<double>(uint32_t x) { return (double)x * 0x1p-32; }
template <> __device__ __forceinline__ float u01<float>(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }
template <typename R> __device__ __forceinline__ R uone(uint32_t x);
template <> __device__ __forceinline__ double uone<double>(uint32_t x) { return (double)x * 0x1p-32 * 2.0 + (-1.0); }
template <> __device__ __forceinline__ float uone<float>(uint32_t x) { return (float)(x >> 8) * 0x1p-23f - 1.0f; }
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
    unsigned long long* pthr;
    double* tal;   // rows x cols (row-major in shared: r * cols + c)
    double* dif;   // rows x (cols + 1) difference array
};

// Shared layout sizes (bytes); tables first, tally last.
template <typename R>
__host__ __device__ inline size_t smemTableBytes(int nw, int np) {
    size_t b = 2 * sizeof(R) * (size_t)nw * np;
    b = (b + 15) & ~(size_t)15;
    b += sizeof(unsigned long long) * (size_t)nw * (np + 1);
    return (b + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t smemTallyBytes(int rows, int cols) {
    return sizeof(double) * (size_t)rows * (2 * (size_t)cols + 1);
}

// Tally modes
enum { TM_SHARED = 0, TM_GLOBAL = 1 };

// Hard cap on events one thread processes in one launch (a guard: a
// phonon that reaches it is killed and flagged non-finite).
constexpr int MAX_EVENTS_PER_LAUNCH = 1 << 22;

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

template <typename R, int TM>
struct Tally {
    const Params<R>* P;
    const Smem<R>* sm;
    int rows;
    // amount per metre of flight, rows entries: Temp sign/v; Flux sign*d
    R rho[4];

    __device__ __forceinline__ void addCell(int col, R t) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (r < rows) {
                if (TM == TM_SHARED) atomicAdd(&sm->tal[r * P->cols + col], (double)(rho[r] * t));
                else atomicAdd(&P->tally[(size_t)col * rows + r], (double)(rho[r] * t));
            }
        }
    }
    // interior cells [c0, c1) of a 1-D walk each get path length t
    __device__ __forceinline__ void addRange(int c0, int c1, int stride, R t) {
        if (c0 >= c1) return;
        if (TM == TM_SHARED && stride == 1) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (r < rows) {
                    double v = (double)(rho[r] * t);
                    atomicAdd(&sm->dif[r * (P->cols + 1) + c0], v);
                    atomicAdd(&sm->dif[r * (P->cols + 1) + c1], -v);
                }
            }
        } else {
            for (int c = c0; c < c1; ++c) addCell(c * stride, t);
        }
    }
};

template <typename R>
__device__ __forceinline__ void reducedVel(const SdomD<R>& S, const R d[3], R a[3]) {
    R m[3];
    rotate(S.Minv, d, m);
    a[0] = S.S[0] * m[0]; a[1] = S.S[1] * m[1]; a[2] = S.S[2] * m[2];
}

template <typename R>
__device__ __forceinline__ R clamp01(R x) { return fmin(fmax(x, R(0)), R(1)); }

// 1-D flight along axis K (the only axis with cells): closed form of
// montecarlo/field.cpp:187-223 -- partial first and last cells, full
// interior cells through the difference array.
template <typename R, int TM, int K>
__device__ __forceinline__ void fly1d(Phn<R>& ph, const SdomD<R>& S, const R a[3], R s, Tally<R, TM>& T) {
    const int cb = S.colbeg;
    const int b = ph.idx[K];
    const int n = S.shape[K];
    const R u = (R)b + ph.off[K] + s * a[K];
    int e = (int)floor(u);
    e = min(max(e, 0), n - 1);
    const int stride = (K == 0) ? 1 : (K == 1 ? S.shape[0] : S.shape[0] * S.shape[1]);
    if (e == b) {
        T.addCell(cb + b * stride, s);
    } else {
        const R inva = R(1) / fabs(a[K]);
        const int lo = min(b, e), hi = max(b, e);
        const R tfirst = (e > b ? (R(1) - ph.off[K]) : ph.off[K]) * inva;
        const R tlast = s - tfirst - (R)(hi - lo - 1) * inva;
        T.addCell(cb + b * stride, tfirst);
        T.addCell(cb + e * stride, fmax(tlast, R(0)));
        if (stride == 1) T.addRange(cb + lo + 1, cb + hi, 1, inva);
        else for (int c = lo + 1; c < hi; ++c) T.addCell(cb + c * stride, inva);
    }
    ph.idx[K] = e;
    ph.off[K] = clamp01(u - (R)e);
#pragma unroll
    for (int j = 0; j < 3; ++j)
        if (j != K) ph.off[j] = clamp01(ph.off[j] + s * a[j]);
}

// Flight of path length s from the current cell, tallied cell by cell
// (Field::accumulate, montecarlo/field.cpp:160-288, as a cell walk).
template <typename R, int TM>
__device__ __forceinline__ void fly(Phn<R>& ph, const SdomD<R>& S, const R a[3], R s, Tally<R, TM>& T) {
    const int acc = S.accum;
    const int cb = S.colbeg;
    if (acc < -1) {
        // no tally: move only
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R u = (R)ph.idx[k] + ph.off[k] + s * a[k];
            int i = (int)floor(u);
            i = min(max(i, 0), S.shape[k] - 1);
            ph.idx[k] = i;
            ph.off[k] = clamp01(u - (R)i);
        }
        return;
    }
    if (acc == -1) {
        T.addCell(cb, s);
#pragma unroll
        for (int k = 0; k < 3; ++k) ph.off[k] = clamp01(ph.off[k] + s * a[k]);
        return;
    }
    if (acc == 0) { fly1d<R, TM, 0>(ph, S, a, s, T); return; }
    if (acc == 1) { fly1d<R, TM, 1>(ph, S, a, s, T); return; }
    if (acc == 2) { fly1d<R, TM, 2>(ph, S, a, s, T); return; }
    // 2-D / 3-D: walk the cells (Amanatides-Woo)
    R rem = s;
    const int s0 = S.shape[0], s01 = S.shape[0] * S.shape[1];
    for (int guard = 0; guard < 3 * MAX_SHAPE + 4; ++guard) {
        R tmin = rem;
        int ax = -1;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R t = tmin;
            if (a[k] > R(0) && ph.idx[k] < S.shape[k] - 1) t = (R(1) - ph.off[k]) / a[k];
            else if (a[k] < R(0) && ph.idx[k] > 0) t = ph.off[k] / (-a[k]);
            if (t < tmin) { tmin = t; ax = k; }
        }
        tmin = fmax(tmin, R(0));
        T.addCell(cb + ph.idx[0] + ph.idx[1] * s0 + ph.idx[2] * s01, tmin);
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
__device__ __forceinline__ void logEvent(const Params<R>& P, const Phn<R>& ph, const SdomD<R>& Sb,
                                         int sBefore, int face, int sAfter, double xEnd[3], double time,
                                         int cellEnd) {
    if (P.log == nullptr || (long long)ph.id >= P.logn) return;
    long long i = ph.nloop;
    if (i >= P.logcap) return;
    double* r = P.log + ((long long)ph.id * P.logcap + i) * 12;
    r[0] = (double)ph.nloop; r[1] = sBefore; r[2] = face; r[3] = sAfter; r[4] = cellEnd;
    r[5] = xEnd[0]; r[6] = xEnd[1]; r[7] = xEnd[2]; r[8] = time; r[9] = (double)ph.nscat;
    r[10] = ph.w; r[11] = ph.p;
    atomicMax(&P.logcount[ph.id], (int)(i + 1));
}

// -------------------------------------------------------------- emission
// FieldProblem::solve emission part (montecarlo/problem.cpp:386-399) and
// Emitter::emit (montecarlo/boundary.cpp:378-385).
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
    for (int k = 0; k < 3; ++k) {
        int i = (int)floor(u[k]);
        i = min(max(i, 0), S.shape[k] - 1);
        ph.idx[k] = i;
        ph.off[k] = u[k] - (R)i;
        ph.d[k] = dir[k];
    }
    // drawScatNext (montecarlo/material.cpp:287-296)
    R vt = P.vt[ph.w * P.np + ph.p];
    R dist = R(0);
    for (int guard = 0; guard < 64 && dist < Lim<R>::tiny(); ++guard) dist = vt * neglog1m(g.next(), R(0));
    ph.scatNext = dist;
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
template <typename R, bool REPLAY, bool LOG, int TM>
__global__ void __launch_bounds__(256) k_advance(Params<R> P) {
    extern __shared__ __align__(16) unsigned char smraw[];
    Smem<R> sm;
    {
        size_t nt = (size_t)P.nw * P.np;
        sm.vel = reinterpret_cast<R*>(smraw);
        sm.vt = sm.vel + nt;
        size_t off = (2 * sizeof(R) * nt + 15) & ~(size_t)15;
        sm.wthr = reinterpret_cast<unsigned long long*>(smraw + off);
        sm.pthr = sm.wthr + P.nw;
        size_t tb = smemTableBytes<R>(P.nw, P.np);
        sm.tal = reinterpret_cast<double*>(smraw + tb);
        sm.dif = sm.tal + (size_t)P.rows * P.cols;
        for (size_t i = threadIdx.x; i < nt; i += blockDim.x) {
            sm.vel[i] = P.vel[i];
            sm.vt[i] = P.vt[i];
            sm.pthr[i] = P.pthr[i];
        }
        for (int i = threadIdx.x; i < P.nw; i += blockDim.x) sm.wthr[i] = P.wthr[i];
        if (TM == TM_SHARED) {
            size_t nz = (size_t)P.rows * (2 * P.cols + 1);
            for (size_t i = threadIdx.x; i < nz; i += blockDim.x) sm.tal[i] = 0.0;
        }
    }
    __syncthreads();

    const unsigned long long n = *P.nlive_in;
    const int keff = min(P.ksteps, P.nsteps - P.step0);
    const R window = (R)keff * P.dt;
    const R invdt = R(1) / P.dt;
    const bool last = (P.step0 + keff >= P.nsteps);
    double csum[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned long long cSteps = 0, cEvents = 0, cScat = 0, cEsc = 0, cHor = 0, cMaxs = 0, cMaxl = 0,
                       cAbs = 0, cBad = 0;
    const int lane = threadIdx.x & 31;

    Tally<R, TM> T;
    T.P = &P;
    T.sm = &sm;
    T.rows = P.rows;

    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long i = base + threadIdx.x;
        bool alive = false;
        Phn<R> ph;
        typename Vec4<R>::T A0, A1;
        uint4 A2;
        if (i < n) {
            ld4(P.P0in + i, A0);
            ld4(P.P1in + i, A1);
            A2 = __ldcs(P.P2in + i);
            unpackCell(A2.x, ph.s, ph.idx);
            ph.off[0] = A0.x; ph.off[1] = A0.y; ph.off[2] = A0.z; ph.scatNext = A0.w;
            ph.d[0] = A1.x; ph.d[1] = A1.y; ph.d[2] = A1.z;
            ph.id = realToId<R>(A1.w);
            ph.w = (int)(A2.y & 0xFFFFu);
            ph.p = (int)((A2.y >> 16) & 0xFFu);
            ph.neg = (A2.y >> 24) & 1u;
            ph.nscat = A2.z;
            ph.nloop = A2.w;
            alive = true;

            Rng<REPLAY> g;
            g.init(P.key0, P.key1, ph.id, &P);
            R budget = window;
            const SdomD<R>* S = &P.sd[ph.s];
            R a[3];
            reducedVel(*S, ph.d, a);
            R v = sm.vel[ph.w * P.np + ph.p];
            R sg = ph.neg ? R(-1) : R(1);
            int stopReason = 0;  // 0 alive, else counter id
            int nev = 0;
            T.rho[1] = T.rho[2] = T.rho[3] = R(0);
            for (;;) {
                // Subdomain::advect: nearest approaching face vs free path
                R sev = ph.scatNext;
                int face = -1;
#pragma unroll
                for (int f = 0; f < 6; ++f) {
                    const int k = f % 3;
                    R dist;
                    bool app;
                    if (f < 3) { app = a[k] < R(0); dist = (-(R)ph.idx[k] - ph.off[k]) / a[k]; }
                    else { app = a[k] > R(0); dist = (((R)(S->shape[k] - ph.idx[k])) - ph.off[k]) / a[k]; }
                    if (app && dist < sev) { sev = dist; face = f; }
                }
                const R tev = sev / v;
                const bool event = tev <= budget;
                const R s = event ? sev : budget * v;
                // tally amounts per metre (montecarlo/problem.cpp:473-544)
                if (P.problem == P_TEMP) { T.rho[0] = sg / v; }
                else if (P.problem == P_FLUX) { T.rho[0] = sg * ph.d[0]; T.rho[1] = sg * ph.d[1]; T.rho[2] = sg * ph.d[2]; }
                else { T.rho[0] = sg / v; T.rho[1] = sg * ph.d[0]; T.rho[2] = sg * ph.d[1]; T.rho[3] = sg * ph.d[2]; }
                const int sBefore = ph.s;
                int cellEnd = 0;
#pragma unroll
                for (int r = 0; r < 4; ++r) csum[r] += (double)(T.rho[r] * s);
                fly<R, TM>(ph, *S, a, s, T);
                if (LOG) cellEnd = ph.idx[0] + ph.idx[1] * S->shape[0] + ph.idx[2] * S->shape[0] * S->shape[1];
                ph.scatNext -= s;
                if (ph.scatNext < Lim<R>::tiny()) ph.scatNext = R(0);
                if (!event) {
                    budget = R(0);
                    if (!(ph.scatNext == ph.scatNext)) stopReason = C_BAD;
                    break;
                }
                budget -= tev;
                if (sev < -S->eps) {
                    stopReason = C_ESCAPES;
                    if (LOG) {
                        double x[3]; physPos(*S, ph, x);
                        logEvent(P, ph, *S, sBefore, -3, sBefore, x,
                                 (double)P.step0 * (double)P.dt + (double)(window - budget), cellEnd);
                    }
                    break;
                }
                double xe[3];
                if (LOG) physPos(*S, ph, xe);
                g.setEvent(ph.nloop + 1);
                bool dirChanged = false;
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
                        dirChanged = true;
                        break;
                    }
                    case F_DIFF: {  // montecarlo/boundary.cpp:308-312
                        R vv[3];
                        drawAniso<R>(g, false, vv);
                        rotate(F.rot, vv, ph.d);
                        normalize(ph.d);
                        ph.nscat++;
                        dirChanged = true;
                        break;
                    }
                    case F_ISOT:  // montecarlo/boundary.cpp:455-460
                        stopReason = C_ABSORBED;
                        break;
                    case F_PERI:   // montecarlo/boundary.cpp:516-522
                    case F_INTER: {  // montecarlo/boundary.cpp:349-359 (single pair)
                        if (F.to < 0) { stopReason = C_ESCAPES; break; }
                        R u[3], u2[3];
                        for (int j = 0; j < 3; ++j) u[j] = (R)ph.idx[j] + ph.off[j];
                        rotate(F.A, u, u2);
                        for (int j = 0; j < 3; ++j) u2[j] += F.b[j];
                        ph.s = F.to;
                        S = &P.sd[ph.s];
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
                            ph.off[j] = fmin(fmax(u2[j] - (R)ii, R(0)), R(1));
                        }
                        if (F.kind == F_PERI && !F.ident) {
                            R dd[3] = {ph.d[0], ph.d[1], ph.d[2]};
                            rotate(F.Rd, dd, ph.d);
                            normalize(ph.d);
                        }
                        dirChanged = true;
                        break;
                    }
                    }
                } else {
                    // Material::scatter (montecarlo/material.cpp:298-303)
                    uint32_t x1 = g.next(), x2 = g.next();
                    ph.w = searchThr(sm.wthr, P.nw, x1);
                    ph.p = searchBranch(sm.pthr + ph.w * P.np, P.np, x2);
                    drawIso<R>(g, ph.d);
                    normalize(ph.d);
                    ph.nscat++;
                    R vt = sm.vt[ph.w * P.np + ph.p];
                    R dist = R(0);
                    for (int guard = 0; guard < 64 && dist < Lim<R>::tiny(); ++guard)
                        dist = vt * neglog1m(g.next(), R(0));
                    ph.scatNext = dist;
                    v = sm.vel[ph.w * P.np + ph.p];
                    dirChanged = true;
                    ++cScat;
                }
                ++cEvents;
                if (LOG) {
                    logEvent(P, ph, P.sd[sBefore], sBefore, face, ph.s, xe,
                             (double)P.step0 * (double)P.dt + (double)(window - budget), cellEnd);
                }
                ph.nloop++;
                if (REPLAY && g.exhausted()) { stopReason = C_REPLAY_EXHAUSTED; break; }
                if (stopReason) break;
                if ((long long)ph.nscat >= P.maxscat) { stopReason = C_MAXSCAT; break; }
                if ((long long)ph.nloop >= P.maxloop) { stopReason = C_MAXLOOP; break; }
                if (++nev >= MAX_EVENTS_PER_LAUNCH) { stopReason = C_BAD; break; }
                if (dirChanged) reducedVel(*S, ph.d, a);
            }
            if (REPLAY) g.save();
            // phonon-steps processed in this window
            if (stopReason == 0) {
                cSteps += keff;
                if (last) {
                    stopReason = C_HORIZON;
                    if (LOG) {
                        double x[3]; physPos(*S, ph, x);
                        int ce = ph.idx[0] + ph.idx[1] * S->shape[0] + ph.idx[2] * S->shape[0] * S->shape[1];
                        logEvent(P, ph, *S, ph.s, -2, ph.s, x, (double)P.nsteps * (double)P.dt, ce);
                    }
                }
            } else {
                R el = window - budget;
                long long st = (long long)ceil(el * invdt);
                st = st < 1 ? 1 : (st > keff ? keff : st);
                cSteps += st;
            }
            switch (stopReason) {
            case 0: break;
            case C_ESCAPES: ++cEsc; break;
            case C_HORIZON: ++cHor; break;
            case C_MAXSCAT: ++cMaxs; break;
            case C_MAXLOOP: ++cMaxl; break;
            case C_ABSORBED: ++cAbs; break;
            case C_REPLAY_EXHAUSTED: atomicOr(P.status, (unsigned)S_REPLAY_EXHAUSTED); break;
            default: ++cBad; atomicOr(P.status, (unsigned)S_NONFINITE); break;
            }
            alive = (stopReason == 0);
            if (alive) {
                A0.x = ph.off[0]; A0.y = ph.off[1]; A0.z = ph.off[2]; A0.w = ph.scatNext;
                A1.x = ph.d[0]; A1.y = ph.d[1]; A1.z = ph.d[2];
                A2.x = packCell(ph.s, ph.idx);
                A2.y = packProp(ph.w, ph.p, ph.neg);
                A2.z = ph.nscat;
                A2.w = ph.nloop;
            }
        }
        // fused compaction: one atomic per warp
        const unsigned mask = __ballot_sync(0xFFFFFFFFu, alive);
        unsigned long long wbase = 0;
        if (lane == 0 && mask) wbase = atomicAdd(P.nlive_out, (unsigned long long)__popc(mask));
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
        if (alive) {
            const unsigned long long o = wbase + __popc(mask & ((1u << lane) - 1u));
            st4(P.P0out + o, A0);
            st4(P.P1out + o, A1);
            __stcs(P.P2out + o, A2);
        }
    }

    // counters: warp reduce, one atomic per warp
    unsigned long long cs[9] = {cSteps, cEvents, cScat, cEsc, cHor, cMaxs, cMaxl, cAbs, cBad};
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
        double x = csum[r];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if (lane == 0 && r < P.rows && x != 0.0) atomicAdd(&P.csum[r], x);
    }

    if (TM == TM_SHARED) {
        __syncthreads();
        // difference array -> cell values (one warp per row), then flush
        const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        for (int r = warp; r < P.rows; r += nwarps) {
            double carry = 0.0;
            double* dr = sm.dif + r * (P.cols + 1);
            for (int c0 = 0; c0 < P.cols; c0 += 32) {
                int c = c0 + lane;
                double x = c < P.cols ? dr[c] : 0.0;
                for (int o = 1; o < 32; o <<= 1) {
                    double y = __shfl_up_sync(0xFFFFFFFFu, x, o);
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
            double x = sm.tal[q];
            if (x != 0.0) {
                const int r = q / P.cols, c = q - r * P.cols;
                atomicAdd(&P.tally[(size_t)c * P.rows + r], x);
            }
        }
    }
}

}  // namespace mcg
