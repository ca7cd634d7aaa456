// mc_oracle.cpp -- CPU oracle: FP64 restatement of montecarlocpp's field solve.
//
// TEST INFRASTRUCTURE ONLY (see mc_oracle.h). Each function cites the
// reference file:line it restates. Parity against the original binary is
// unpinned (Eigen 3 and Boost are not available to build it); the choices
// made where the reference's behaviour lives inside those libraries are:
//   * uniform_01<double> / uniform_real_distribution(-1,1) on a 32-bit
//     engine: u = x / 2^32 and 2u - 1 (one engine word each);
//   * discrete_distribution: inverse-CDF search on the FP64 cumulative table
//     (one uniform for the frequency bin, one for the branch);
//   * Quaternion::FromTwoVectors(z, n): the standard half-angle quaternion
//     about z x n; for n = -z the rotation by pi about x.
//   * the three uniforms of a volume position are consumed x, y, z in order.
// Build with -ffp-contract=off so x86 and Arm give identical bits.

#include "mc_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <random>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// montecarlo/constants.h:17-19
const double PI = 3.141592653589793;
const double HBAR = 1.054560652927e-034;
const double KB = 1.380648e-023;
const double DMIN = std::numeric_limits<double>::min();
const double DEPS = std::numeric_limits<double>::epsilon();
const double TWO_M32 = 1.0 / 4294967296.0;

// ----------------------------------------------------------------- vectors
struct V3 {
    double v[3];
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};
inline V3 mk(double a, double b, double c) { V3 r; r[0] = a; r[1] = b; r[2] = c; return r; }
inline V3 z3() { return mk(0., 0., 0.); }
inline V3 add(const V3& a, const V3& b) { return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline V3 sub(const V3& a, const V3& b) { return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline V3 scl(double s, const V3& a) { return mk(a[0] * s, a[1] * s, a[2] * s); }
inline double dot(const V3& a, const V3& b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline V3 cross(const V3& a, const V3& b) {
    return mk(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline double norm(const V3& a) { return std::sqrt(dot(a, a)); }
inline V3 normalized(const V3& a) {
    double z = dot(a, a);
    if (z > 0.) { double s = std::sqrt(z); return mk(a[0] / s, a[1] / s, a[2] / s); }
    return a;
}
struct M3 {
    double m[9];  // row-major
    double operator()(int r, int c) const { return m[3 * r + c]; }
    double& operator()(int r, int c) { return m[3 * r + c]; }
};
inline M3 ident() { M3 r; for (int i = 0; i < 9; ++i) r.m[i] = (i % 4 == 0) ? 1. : 0.; return r; }
inline V3 mul(const M3& a, const V3& x) {
    return mk((a(0, 0) * x[0] + a(0, 1) * x[1]) + a(0, 2) * x[2],
              (a(1, 0) * x[0] + a(1, 1) * x[1]) + a(1, 2) * x[2],
              (a(2, 0) * x[0] + a(2, 1) * x[1]) + a(2, 2) * x[2]);
}
inline V3 col(const M3& a, int c) { return mk(a(0, c), a(1, c), a(2, c)); }
inline M3 transpose(const M3& a) { M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r(i, j) = a(j, i); return r; }
inline double det(const M3& a) {
    return a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) -
           a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
           a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
}
inline M3 inverse(const M3& a) {
    // cofactor inverse of a 3x3 matrix
    double d = det(a);
    M3 r;
    r(0, 0) = (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) / d;
    r(0, 1) = (a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2)) / d;
    r(0, 2) = (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1)) / d;
    r(1, 0) = (a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2)) / d;
    r(1, 1) = (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0)) / d;
    r(1, 2) = (a(0, 2) * a(1, 0) - a(0, 0) * a(1, 2)) / d;
    r(2, 0) = (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0)) / d;
    r(2, 1) = (a(0, 1) * a(2, 0) - a(0, 0) * a(2, 1)) / d;
    r(2, 2) = (a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0)) / d;
    return r;
}

// Rotation taking z-hat to n (montecarlo/boundary.cpp:33-37,
// montecarlo/subdomain.cpp:26-30): half-angle quaternion about z x n,
// converted to a matrix with the standard formula.
M3 rotZTo(const V3& nIn) {
    V3 v0 = mk(0., 0., 1.);
    V3 v1 = normalized(nIn);
    double c = dot(v1, v0);
    double qw, qx, qy, qz;
    if (c < -1. + 1e-12) {
        // antiparallel: rotation by pi about x (the reference's axis comes
        // from an SVD inside Eigen and is unpinned)
        qw = 0.; qx = 1.; qy = 0.; qz = 0.;
    } else {
        V3 axis = cross(v0, v1);
        double s = std::sqrt((1. + c) * 2.);
        double invs = 1. / s;
        qx = axis[0] * invs; qy = axis[1] * invs; qz = axis[2] * invs;
        qw = s * 0.5;
    }
    double tx = 2. * qx, ty = 2. * qy, tz = 2. * qz;
    double twx = tx * qw, twy = ty * qw, twz = tz * qw;
    double txx = tx * qx, txy = ty * qx, txz = tz * qx;
    double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
    M3 r;
    r(0, 0) = 1. - (tyy + tzz); r(0, 1) = txy - twz;        r(0, 2) = txz + twy;
    r(1, 0) = txy + twz;        r(1, 1) = 1. - (txx + tzz); r(1, 2) = tyz - twx;
    r(2, 0) = txz - twy;        r(2, 1) = tyz + twx;        r(2, 2) = 1. - (txx + tyy);
    return r;
}

// --------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with a
// Weyl-sequence key schedule.
void philox(const uint32_t ctrIn[4], const uint32_t keyIn[2], uint32_t out[4]) {
    uint32_t c0 = ctrIn[0], c1 = ctrIn[1], c2 = ctrIn[2], c3 = ctrIn[3];
    uint32_t k0 = keyIn[0], k1 = keyIn[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// ---------------------------------------------------------- uniform source
struct Source {
    int kind = ORC_RNG_PHILOX;
    std::mt19937* mt = nullptr;
    uint32_t key[2] = {0, 0};
    uint32_t id = 0, event = 0, block = 0;
    uint32_t buf[4];
    int lane = 4;
    const uint32_t* rw = nullptr;
    int64_t rpos = 0, rend = 0;
    bool exhausted = false;
    uint32_t* rec = nullptr;
    int64_t reccount = 0;
    long reccap = 0;

    void setEvent(uint32_t e) { event = e; block = 0; lane = 4; }
    uint32_t word() {
        uint32_t x = 0;
        if (kind == ORC_RNG_MT_THREADS) {
            x = (uint32_t)(*mt)();
        } else if (kind == ORC_RNG_PHILOX) {
            if (lane == 4) {
                uint32_t ctr[4] = {id, event, block, 0u};
                philox(ctr, key, buf);
                ++block;
                lane = 0;
            }
            x = buf[lane++];
        } else {
            if (rpos < rend) x = rw[rpos++];
            else { exhausted = true; x = 0x80000000u; }
        }
        if (rec) {
            if (reccount < reccap) rec[reccount] = x;
            ++reccount;
        }
        return x;
    }
    // boost uniform_01<double> on a 32-bit engine: x / 2^32, in [0, 1)
    double u01() { return (double)word() * TWO_M32; }
    // boost uniform_real_distribution<double>(-1, 1): in [-1, 1)
    double uOne() { return (double)word() * TWO_M32 * 2.0 + (-1.0); }
};

// --------------------------------------------------------------- material
struct Dist {
    long nw = 0, np = 0;
    std::vector<double> wcdf;  // nw
    std::vector<double> pcdf;  // nw x np
    // montecarlo/material.cpp:123-141 builds a two-level discrete
    // distribution: bin by row sum, then branch within the bin.
    void build(const std::vector<double>& pdf, long nw_, long np_) {
        nw = nw_; np = np_;
        std::vector<double> rowSum(nw);
        for (long w = 0; w < nw; ++w) {
            double s = 0.;
            for (long p = 0; p < np; ++p) s += pdf[w * np + p];
            rowSum[w] = s;
        }
        wcdf.assign(nw, 0.);
        double acc = 0.;
        std::vector<double> pre(nw);
        for (long w = 0; w < nw; ++w) { acc += rowSum[w]; pre[w] = acc; }
        for (long w = 0; w < nw; ++w) wcdf[w] = pre[w] / acc;
        pcdf.assign(nw * np, 1.);
        for (long w = 0; w < nw; ++w) {
            if (!(rowSum[w] > 0.)) continue;
            double a = 0.;
            std::vector<double> pp(np);
            for (long p = 0; p < np; ++p) { a += pdf[w * np + p]; pp[p] = a; }
            for (long p = 0; p < np; ++p) pcdf[w * np + p] = pp[p] / a;
        }
    }
    static long pick(const double* cdf, long n, double u) {
        // first index with u < cdf[i]
        long lo = 0, hi = n;  // answer in [lo, hi)
        while (lo < hi) {
            long mid = (lo + hi) / 2;
            if (u < cdf[mid]) hi = mid; else lo = mid + 1;
        }
        return lo < n ? lo : n - 1;
    }
    // montecarlo/material.cpp:143-147
    void draw(double u1, double u2, long& w, long& p) const {
        w = pick(wcdf.data(), nw, u1);
        p = pick(pcdf.data() + w * np, np, u2);
    }
};

}  // namespace

struct orc_material {
    long nw = 0, np = 0;
    double T = 0., k = 0.;
    std::vector<double> omega, tau, vel;  // tau, vel: nw x np row-major
    Dist energy, flux, scat;
    double energySum = 0., fluxSum = 0., scatSum = 0.;

    double velOf(long w, long p) const { return vel[w * np + p]; }
    double tauOf(long w, long p) const { return tau[w * np + p]; }
};

namespace {

// montecarlo/material.cpp:154-234
orc_material* buildMaterial(const double* disp, long nw, long np,
                            const double* relax, double T) {
    orc_material* m = new orc_material;
    m->nw = nw; m->np = np; m->T = T;
    m->omega.resize(nw);
    std::vector<double> domega(nw), dos(nw * np);
    m->vel.resize(nw * np);
    long ncol = 2 + 2 * np;
    for (long w = 0; w < nw; ++w) {
        m->omega[w] = disp[w * ncol + 0];
        domega[w] = disp[w * ncol + 1];
        for (long p = 0; p < np; ++p) {
            m->vel[w * np + p] = disp[w * ncol + 2 + 2 * p];
            dos[w * np + p] = disp[w * ncol + 3 + 2 * p];
        }
    }
    // relaxation times: two Matthiessen terms c0 w^c1 T^c2 exp(-c3/T)
    m->tau.assign(nw * np, 0.);
    for (long p = 0; p < np; ++p) {
        std::vector<double> tauinv(nw, 0.);
        for (int j = 0; j < 2; ++j) {
            const double* c = relax + p * 8 + 4 * j;
            if (c[0] <= DMIN) continue;
            double tp = std::pow(T, c[2]) ;
            double ex = std::exp(-c[3] / T);
            for (long w = 0; w < nw; ++w)
                tauinv[w] += c[0] * std::pow(m->omega[w], c[1]) * tp * ex;
        }
        for (long w = 0; w < nw; ++w) m->tau[w * np + p] = 1. / tauinv[w];
    }
    // dE/dT (montecarlo/material.cpp:208-217)
    std::vector<double> dedT(nw);
    double xs = HBAR / (KB * T);
    for (long w = 0; w < nw; ++w) {
        double x = xs * m->omega[w];
        double q = x / (2. * std::sinh(x / 2.));
        dedT[w] = KB * (std::fabs(x) < DEPS ? 1. - x * x / 12. : q * q);
    }
    std::vector<double> epdf(nw * np), fpdf(nw * np), spdf(nw * np);
    double es = 0., fs = 0., ss = 0., k = 0.;
    for (long w = 0; w < nw; ++w)
        for (long p = 0; p < np; ++p) {
            long i = w * np + p;
            epdf[i] = dedT[w] * dos[i] * domega[w];
            fpdf[i] = m->vel[i] * epdf[i];
            spdf[i] = epdf[i] / m->tau[i];
            es += epdf[i]; fs += fpdf[i]; ss += spdf[i];
            k += m->tau[i] * (m->vel[i] * m->vel[i]) * epdf[i];
        }
    m->energy.build(epdf, nw, np);
    m->flux.build(fpdf, nw, np);
    m->scat.build(spdf, nw, np);
    m->energySum = es; m->fluxSum = fs; m->scatSum = ss;
    m->k = k / 3.;
    return m;
}

bool readNumbers(const char* path, std::vector<double>& out) {
    std::ifstream f(path);
    if (!f) return false;
    double x;
    while (f >> x) out.push_back(x);
    return true;
}

// ----------------------------------------------------------------- geometry
struct Face {
    int kind = ORC_SPEC;
    int shape = 0;     // 0 Parallelogram, 1 Triangle, 2 Polygon
    V3 n, o, si, sj;   // inward normal, face origin, shape vectors
    std::vector<V3> verts;     // Polygon: the N - 1 vertices relative to o
    std::vector<double> pcdf;  // Polygon: cumulative triangle areas
    double off = 0.;   // plane offset: signed distance = n.x + off
    double T = 0.;
    double area = 0.;
    M3 refl, rot;      // Spec reflection, z->n rotation
    // Peri
    int pairS = -1, pairF = -1;
    M3 prot;
    V3 ptransl;
    // Inter
    std::vector<std::pair<int, int> > inter;
};

struct Sdom {
    int shapeKind = ORC_PARALLELEPIPED;
    V3 o;
    M3 M, inv;
    long div[3], shape[3], max[3];
    int accum = -1;
    double eps = 0., vol = 0.;
    std::vector<Face> f;
    V3 gradT;
    M3 rot;
    long colbeg = -1;
    std::vector<V3> mcol;      // Prism / Pyramid: the N matrix columns
    std::vector<double> vcdf;  // Prism / Pyramid: volDist cumulative weights
    double emitWeight() const { return 2. * vol * norm(gradT); }
};

struct Emitter {
    int sdom;
    int face;  // -1: volume emitter
};

}  // namespace

struct orc_domain {
    std::vector<Sdom> sd;
    std::vector<Emitter> em;
    long cols = 0;

    double emitWeight(const Emitter& e) const {
        const Sdom& s = sd[e.sdom];
        if (e.face < 0) return s.emitWeight();
        const Face& f = s.f[e.face];
        return f.area * std::fabs(f.T);  // montecarlo/boundary.cpp:413-416
    }
    bool isInside(int s, const V3& x) const {
        // montecarlo/subdomain.cpp:108-116
        const Sdom& d = sd[s];
        for (size_t i = 0; i < d.f.size(); ++i)
            if (dot(d.f[i].n, x) + d.f[i].off < -d.eps) return false;
        return true;
    }
};

namespace {

// Discrete distribution over non-negative weights as its normalised
// cumulative table (drawn with Dist::pick).
std::vector<double> cdfOf(const std::vector<double>& w) {
    std::vector<double> c(w.size());
    double acc = 0.;
    for (size_t i = 0; i < w.size(); ++i) { acc += w[i]; c[i] = acc; }
    for (size_t i = 0; i < w.size(); ++i) c[i] /= acc;
    return c;
}

// Boundary(o, shape) (montecarlo/boundary.cpp:50-54) with the shape's
// normal and area: Parallelogram (montecarlo/boundary.cpp:121-152),
// Triangle (154-186), Polygon<N> (188-258).
Face makeFace(int kind, double T, const V3& o, int shape, const V3& si, const V3& sj,
              const std::vector<V3>& verts = std::vector<V3>()) {
    Face f;
    f.kind = kind;
    f.T = T;
    f.o = o;
    f.shape = shape;
    f.si = si;
    f.sj = sj;
    if (shape == 2) {
        f.verts = verts;
        std::vector<double> a;
        // montecarlo/boundary.cpp:199-210: triangles (v_n, v_n+1), n < N - 2
        for (size_t k = 0; k + 1 < verts.size(); ++k) a.push_back(norm(cross(verts[k], verts[k + 1])) / 2.);
        double tot = 0.;
        for (double x : a) tot += x;
        f.area = tot;
        f.pcdf = cdfOf(a);
        f.n = normalized(cross(verts[0], verts[1]));
    } else {
        V3 cr = cross(si, sj);
        f.n = normalized(cr);
        f.area = shape == 1 ? norm(cr) / 2. : norm(cr);
    }
    f.off = -dot(f.n, f.o);
    M3 r = ident();
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) r(a, b) -= 2. * (f.n[a] * f.n[b]);
    f.refl = r;
    f.rot = rotZTo(f.n);
    f.prot = ident();
    f.ptransl = mk(0., 0., 0.);
    return f;
}

// Subdomain::Subdomain (montecarlo/subdomain.cpp:41-71): inverse, shape,
// escape tolerance and accumulation flag of (o, mat, div).
void initSubdomain(Sdom& s, const V3& o, const M3& M, const long div[3]) {
    s.o = o;
    s.M = M;
    s.inv = inverse(s.M);
    double maxn = 0.;
    for (int c = 0; c < 3; ++c) maxn = std::max(maxn, norm(col(s.M, c)));
    s.eps = 100. * DEPS * maxn;
    bool anyNeg = false;
    long npos = 0;
    for (int i = 0; i < 3; ++i) {
        s.div[i] = div[i];
        s.shape[i] = std::max(div[i], 1L);
        s.max[i] = s.shape[i] - 1;
        if (div[i] < 0) anyNeg = true;
        if (div[i] > 0) ++npos;
    }
    if (anyNeg) {
        for (int i = 0; i < 3; ++i) { s.shape[i] = 0; s.max[i] = 0; }
        s.accum = -2;
    } else if (npos == 0) {
        s.accum = -1;
    } else if (npos == 1) {
        int dir = 0;
        for (int i = 1; i < 3; ++i) if (s.div[i] > s.div[dir]) dir = i;
        s.accum = dir;
    } else {
        s.accum = (int)npos + 1;
    }
}

// Faces of each shape in the reference's bdry<I>() order, and the shape's
// volume: Parallelepiped (montecarlo/subdomain.h:145-158), TriangularPrism
// (subdomain.h:224-236), Tetrahedron (subdomain.h:303-314), Prism<N>
// (subdomain.h:386-410 with InitSidesF 458-475; PrismImpl
// montecarlo/subdomain.cpp:376-407) and Pyramid<N> (subdomain.h:524-547
// with InitSidesF 595-613; PyramidImpl subdomain.cpp:409-441). Returns
// false on an invalid description.
bool buildShape(Sdom& s, const orc_sdom& p) {
    const V3 o = mk(p.o[0], p.o[1], p.o[2]);
    const int N = p.ncols;
    std::vector<V3> c(N);
    for (int i = 0; i < N; ++i) c[i] = mk(p.mat[3 * i], p.mat[3 * i + 1], p.mat[3 * i + 2]);
    auto T = [&](int i) { return p.T[i]; };
    auto K = [&](int i) { return p.kind[i]; };
    M3 M;
    long div[3] = {p.div[0], p.div[1], p.div[2]};
    s.shapeKind = p.shape;
    if (p.shape == ORC_PARALLELEPIPED || p.shape == ORC_TRIANGULAR_PRISM || p.shape == ORC_TETRAHEDRON) {
        if (N != 3) return false;
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) M(r, q) = c[q][r];
        initSubdomain(s, o, M, div);
        const double d = det(M);
        if (p.shape == ORC_PARALLELEPIPED) {
            s.vol = d;
            V3 fo[6] = {o, o, o, add(o, c[0]), add(o, c[1]), add(o, c[2])};
            V3 fi[6] = {c[1], c[2], c[0], c[2], c[0], c[1]};
            V3 fj[6] = {c[2], c[0], c[1], c[1], c[2], c[0]};
            for (int k = 0; k < 6; ++k) s.f.push_back(makeFace(K(k), T(k), fo[k], 0, fi[k], fj[k]));
        } else if (p.shape == ORC_TRIANGULAR_PRISM) {
            s.vol = d / 2.;
            s.f.push_back(makeFace(K(0), T(0), o, 0, c[1], c[2]));
            s.f.push_back(makeFace(K(1), T(1), o, 0, c[2], c[0]));
            s.f.push_back(makeFace(K(2), T(2), o, 1, c[0], c[1]));
            s.f.push_back(makeFace(K(3), T(3), add(o, c[0]), 0, c[2], sub(c[1], c[0])));
            s.f.push_back(makeFace(K(4), T(4), add(o, c[2]), 1, c[1], c[0]));
        } else {
            s.vol = d / 6.;
            s.f.push_back(makeFace(K(0), T(0), o, 1, c[1], c[2]));
            s.f.push_back(makeFace(K(1), T(1), o, 1, c[2], c[0]));
            s.f.push_back(makeFace(K(2), T(2), o, 1, c[0], c[1]));
            s.f.push_back(makeFace(K(3), T(3), add(o, c[0]), 1, sub(c[2], c[0]), sub(c[1], c[0])));
        }
    } else if (p.shape == ORC_PRISM || p.shape == ORC_PYRAMID) {
        if (N < 4 || N > ORC_MAX_COLS) return false;
        const bool prism = p.shape == ORC_PRISM;
        // matBase = (col1, col(N-1), col0)
        for (int r = 0; r < 3; ++r) { M(r, 0) = c[1][r]; M(r, 1) = c[N - 1][r]; M(r, 2) = c[0][r]; }
        long d1 = p.div[0] < 0 ? -1 : 0;
        long dv[3] = {d1, d1, d1};
        initSubdomain(s, o, M, dv);
        // volume(mat): col(i) x col(i+1) . col(0) for i < N - 2, / 2 or / 6
        std::vector<double> v(N - 2);
        double vs = 0.;
        for (int i = 0; i < N - 2; ++i) {
            v[i] = dot(cross(c[i], c[i + 1]), c[0]) / (prism ? 2. : 6.);
            vs += v[i];
        }
        s.vol = vs;
        s.vcdf = cdfOf(v);
        s.mcol = c;
        std::vector<V3> bot(c.begin() + 1, c.end());
        s.f.push_back(makeFace(K(0), T(0), o, 2, z3(), z3(), bot));
        int base = 1;
        if (prism) {
            std::vector<V3> top(bot.rbegin(), bot.rend());
            s.f.push_back(makeFace(K(1), T(1), add(o, c[0]), 2, z3(), z3(), top));
            base = 2;
        }
        for (int ind = 0; ind < N; ++ind) {
            V3 pp = ind != 0 ? c[ind] : mk(0., 0., 0.);
            V3 i = prism ? c[0] : (ind != 0 ? sub(c[0], c[ind]) : c[0]);
            V3 j = scl(-1., pp);
            if (ind != N - 1) j = add(j, c[ind + 1]);
            s.f.push_back(makeFace(K(base + ind), T(base + ind), add(o, pp), prism ? 0 : 1, i, j));
        }
    } else {
        return false;
    }
    if (!(s.vol >= DMIN)) return false;
    for (size_t k = 0; k < s.f.size(); ++k) {
        const Face& f = s.f[k];
        if (f.kind < ORC_SPEC || f.kind > ORC_INTER) return false;
        if ((f.kind == ORC_SPEC || f.kind == ORC_DIFF || f.kind == ORC_INTER) && f.T != 0.) return false;
    }
    s.gradT = mk(p.gradT[0], p.gradT[1], p.gradT[2]);
    s.rot = rotZTo(normalized(s.gradT));
    return true;
}

int faceCount(int shape, int ncols) {
    switch (shape) {
    case ORC_PARALLELEPIPED: return 6;
    case ORC_TRIANGULAR_PRISM: return 5;
    case ORC_TETRAHEDRON: return 4;
    case ORC_PRISM: return ncols + 2;
    case ORC_PYRAMID: return ncols + 1;
    default: return 0;
    }
}

// TriangularPrismImpl::drawPos (montecarlo/subdomain.cpp:309-319) and
// TetrahedronImpl::drawPos (subdomain.cpp:348-373) in the unit cell of
// (o, local); the three uniforms are consumed x, y, z.
V3 drawTriPrism(Source& g, const V3& o, const M3& L) {
    double c0 = g.u01(), c1 = g.u01(), c2 = g.u01();
    if (c0 + c1 > 1.) { c0 = 1. - c0; c1 = 1. - c1; }
    return add(o, mul(L, mk(c0, c1, c2)));
}
V3 drawTetra(Source& g, const V3& o, const M3& L) {
    double c0 = g.u01(), c1 = g.u01(), c2 = g.u01();
    if (c0 + c1 > 1.) { c0 = 1. - c0; c1 = 1. - c1; }
    if (c1 + c2 > 1.) {
        double tmp = c2;
        c2 = 1. - c0 - c1;
        c1 = 1. - tmp;
    } else if (c0 + c1 + c2 > 1.) {
        double tmp = c2;
        c2 = c0 + c1 + c2 - 1.;
        c0 = 1. - c1 - tmp;
    }
    return add(o, mul(L, mk(c0, c1, c2)));
}

// EmitSubdomain::drawPos of each shape (ParallelepipedImpl
// montecarlo/subdomain.cpp:275-281; Prism / Pyramid: volDist, then the
// sub-volume of columns (ind + 1, ind + 2, 0), subdomain.cpp:399-407,
// 433-441).
V3 drawVolumePos(const Sdom& s, Source& g) {
    switch (s.shapeKind) {
    case ORC_TRIANGULAR_PRISM: return drawTriPrism(g, s.o, s.M);
    case ORC_TETRAHEDRON: return drawTetra(g, s.o, s.M);
    case ORC_PRISM:
    case ORC_PYRAMID: {
        long ind = Dist::pick(s.vcdf.data(), (long)s.vcdf.size(), g.u01());
        M3 L;
        for (int r = 0; r < 3; ++r) { L(r, 0) = s.mcol[ind + 1][r]; L(r, 1) = s.mcol[ind + 2][r]; L(r, 2) = s.mcol[0][r]; }
        return s.shapeKind == ORC_PRISM ? drawTriPrism(g, s.o, L) : drawTetra(g, s.o, L);
    }
    default: {
        double c0 = g.u01(), c1 = g.u01(), c2 = g.u01();
        return add(s.o, mul(s.M, mk(c0, c1, c2)));
    }
    }
}

// EmitBoundary::drawPos (montecarlo/boundary.cpp:418-421): the face origin
// plus the shape's drawPos.
V3 drawFacePos(const Face& f, Source& g) {
    if (f.shape == 0) {
        double r1 = g.u01(), r2 = g.u01();
        return add(f.o, add(scl(r1, f.si), scl(r2, f.sj)));
    }
    V3 i = f.si, j = f.sj;
    if (f.shape == 2) {
        long n = Dist::pick(f.pcdf.data(), (long)f.pcdf.size(), g.u01());
        i = f.verts[n];
        j = f.verts[n + 1];
    }
    double r1 = g.u01(), r2 = g.u01();
    V3 q = r1 + r2 < 1. ? add(scl(r1, i), scl(r2, j)) : add(scl(1. - r1, i), scl(1. - r2, j));
    return add(f.o, q);
}

// Subdomain::cellVol (ParallelepipedImpl montecarlo/subdomain.cpp:269-273,
// TriangularPrismImpl 283-307, TetrahedronImpl 321-346, PrismImpl and
// PyramidImpl 394-397,428-431).
double cellVolume(const Sdom& s, const long idx[3]) {
    const double sp = (double)(s.shape[0] * s.shape[1] * s.shape[2]);
    if (s.shapeKind == ORC_PARALLELEPIPED) return s.vol / sp;
    if (s.shapeKind == ORC_PRISM || s.shapeKind == ORC_PYRAMID) return s.vol;
    const int dim = s.shapeKind == ORC_TRIANGULAR_PRISM ? 2 : 3;
    double f0 = 1.;
    for (int k = 0; k < dim; ++k) f0 -= (double)idx[k] / (double)s.shape[k];
    if (f0 <= 0.) return 0.;
    double f1 = f0;
    for (int k = 0; k < dim; ++k) f1 -= 1. / (double)s.shape[k];
    if (f1 >= 0.) return s.vol / sp;
    if (dim == 2) {
        double frac = std::pow(f0, 2);
        for (int i = 0; i < 2; ++i) {
            // corners (1,0), (0,1): sign (-1)^1
            double f = f0 - 1. / (double)s.shape[i];
            if (f > 0.) frac += -1. * std::pow(f, 2);
        }
        return s.vol * frac / (2. * (double)s.shape[2]);
    }
    static const int pts[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}};
    double frac = std::pow(f0, 3);
    for (int i = 0; i < 6; ++i) {
        int sum = pts[i][0] + pts[i][1] + pts[i][2];
        double sign = (sum % 2) ? -1. : 1.;
        double f = f0;
        for (int k = 0; k < 3; ++k) f -= (double)pts[i][k] / (double)s.shape[k];
        if (f > 0.) frac += sign * std::pow(f, 3);
    }
    return s.vol * frac / 6.;
}

// ------------------------------------------------------------------ phonon
struct Phonon {
    bool alive = true;
    int sign = 1;
    long w = 0, p = 0;
    V3 pos, dir;
    double time = 0., scatNext = 0.;
    long nscat = 0;
};

// montecarlo/phonon.cpp:95-105 (line origin = pos, direction = dir)
inline void move(Phonon& ph, double d, double vel) {
    ph.scatNext -= d;
    if (ph.scatNext < DMIN) ph.scatNext = 0.;
    ph.time += d / vel;
    ph.pos = add(ph.pos, scl(d, ph.dir));
}

// montecarlo/random.cpp:16-27
inline V3 drawIso(Source& g) {
    double cosT = g.uOne();
    double sinT = std::sqrt(1. - cosT * cosT);
    double phi = PI * g.uOne();
    return mk(sinT * std::cos(phi), sinT * std::sin(phi), cosT);
}

// montecarlo/random.cpp:29-44
inline V3 drawAniso(Source& g, bool bidir) {
    double r = g.uOne();
    int sign = bidir ? (r < 0. ? -1 : 1) : 1;
    double s2 = std::fabs(r);
    double sinT = std::sqrt(s2);
    double cosT = sign * std::sqrt(1. - s2);
    double phi = PI * g.uOne();
    return mk(sinT * std::cos(phi), sinT * std::sin(phi), cosT);
}

// montecarlo/material.cpp:287-296
inline void drawScatNext(const orc_material& m, Phonon& ph, Source& g) {
    double d = 0.;
    double vt = m.velOf(ph.w, ph.p) * m.tauOf(ph.w, ph.p);
    while (d < DMIN) {
        d = vt * -std::log(1. - g.u01());
        if (g.exhausted) break;
    }
    ph.scatNext = d;
}

// ------------------------------------------------------------------- field
struct Field {
    long rows, cols;
    std::vector<double> data;  // column-major rows x cols
    void add(long c, const double* amount, double f) {
        double* col = &data[c * rows];
        for (long r = 0; r < rows; ++r) col[r] += amount[r] * f;
    }
};

inline V3 coordOf(const Sdom& s, const V3& x) {
    // montecarlo/subdomain.cpp:148-151
    V3 c = mul(s.inv, sub(x, s.o));
    return mk((double)s.div[0] * c[0], (double)s.div[1] * c[1], (double)s.div[2] * c[2]);
}
inline void coord2index(const Sdom& s, const V3& c, long idx[3]) {
    // montecarlo/subdomain.cpp:153-159
    for (int i = 0; i < 3; ++i) {
        long v = (long)std::floor(c[i]);
        idx[i] = std::min(std::max(v, 0L), s.max[i]);
    }
}
inline long flatIndex(const Sdom& s, const long idx[3]) {
    return idx[0] + idx[1] * s.shape[0] + idx[2] * s.shape[0] * s.shape[1];
}

// montecarlo/field.cpp:160-288
void accumulate(const orc_domain& D, int si, const V3& bpos, const V3& epos,
                const double* amount, Field& F) {
    const Sdom& s = D.sd[si];
    int flag = s.accum;
    if (flag < -1) return;
    long base = s.colbeg;
    if (flag < 0) { F.add(base, amount, 1.); return; }
    V3 bc = coordOf(s, bpos), ec = coordOf(s, epos), dc = sub(ec, bc);
    long bi[3], ei[3];
    coord2index(s, bc, bi);
    coord2index(s, ec, ei);
    long s1 = 1, s2 = s.shape[0], s3 = s.shape[0] * s.shape[1];
    long stride[3] = {s1, s2, s3};
    if (flag < 3) {
        int d = flag;
        long b = bi[d], e = ei[d];
        if (b == e) { F.add(base + b * stride[d], amount, 1.); return; }
        double inv = 1. / std::fabs(dc[d]);
        long pm;
        if (b < e) {
            F.add(base + b * stride[d], amount, inv * (1 + b - bc[d]));
            F.add(base + e * stride[d], amount, inv * (ec[d] - e));
            pm = 1;
        } else {
            F.add(base + b * stride[d], amount, inv * (bc[d] - b));
            F.add(base + e * stride[d], amount, inv * (1 + e - ec[d]));
            pm = -1;
        }
        for (long n = b + pm; n != e; n += pm) F.add(base + n * stride[d], amount, inv);
        return;
    }
    // 2-D / 3-D: crossing parameters sorted, coincident ones merged
    std::map<double, std::vector<long> > borders;
    for (int d = 0; d < 3; ++d) {
        if (std::fabs(dc[d]) < DMIN) continue;
        long b = bi[d], e = ei[d], pm;
        if (b == e) continue;
        if (b < e) { ++b; ++e; pm = 1; } else { pm = -1; }
        for (long n = b; n != e; n += pm) {
            double param = (n - bc[d]) / dc[d];
            auto it = borders.find(param);
            if (it == borders.end()) it = borders.emplace(param, std::vector<long>(3, 0)).first;
            it->second[d] += pm;
        }
    }
    borders.emplace(1., std::vector<long>(3, 0));
    long idx[3] = {bi[0], bi[1], bi[2]};
    double param = 0.;
    for (auto& kv : borders) {
        F.add(base + flatIndex(s, idx), amount, kv.first - param);
        param = kv.first;
        for (int d = 0; d < 3; ++d) idx[d] += kv.second[d];
    }
}

struct Local {
    Field F;
    orc_stats st;
};

}  // namespace

// =================================================================== C API
extern "C" {

orc_material* orc_material_from_tables(const double* disp, long nw, long np,
                                       const double* relax, double T) {
    return buildMaterial(disp, nw, np, relax, T);
}

orc_material* orc_material_load(const char* disp, const char* relax, double T) {
    // montecarlo/material.cpp:158-186 file formats
    std::vector<double> a, b;
    if (!readNumbers(disp, a) || !readNumbers(relax, b)) return nullptr;
    if (a.size() < 2) return nullptr;
    long nw = (long)a[0], np = (long)a[1];
    if (nw <= 0 || np <= 0) return nullptr;
    if ((long)a.size() < 2 + nw * (2 + 2 * np) || (long)b.size() < 8 * np) return nullptr;
    return buildMaterial(a.data() + 2, nw, np, b.data(), T);
}

void orc_material_free(orc_material* m) { delete m; }

void orc_material_sums(const orc_material* m, double out[4]) {
    out[0] = m->energySum; out[1] = m->fluxSum; out[2] = m->scatSum; out[3] = m->k;
}

void orc_material_draw(const orc_material* m, int which, uint32_t x1,
                       uint32_t x2, long* w, long* p) {
    const Dist& d = which == 0 ? m->energy : (which == 1 ? m->flux : m->scat);
    d.draw((double)x1 * TWO_M32, (double)x2 * TWO_M32, *w, *p);
}

void orc_material_tables(const orc_material* m, double* vel, double* tau) {
    std::memcpy(vel, m->vel.data(), sizeof(double) * m->nw * m->np);
    std::memcpy(tau, m->tau.data(), sizeof(double) * m->nw * m->np);
}

orc_domain* orc_domain_create_shapes(const orc_sdom* s, int ns, const orc_pair* pr, int npairs) {
    if (!s || ns <= 0) return nullptr;
    orc_domain* D = new orc_domain;
    D->sd.resize(ns);
    // construction registers the emitting faces whose weight is nonzero at
    // construction time (montecarlo/subdomain.cpp:205-212)
    std::vector<std::vector<int> > faceEmit(ns);
    for (int i = 0; i < ns; ++i) {
        if (s[i].ncols > ORC_MAX_COLS || faceCount(s[i].shape, s[i].ncols) > ORC_MAX_FACES ||
            !buildShape(D->sd[i], s[i])) {
            delete D;
            return nullptr;
        }
        for (size_t k = 0; k < D->sd[i].f.size(); ++k) {
            const Face& f = D->sd[i].f[k];
            if ((f.kind == ORC_ISOT || f.kind == ORC_PERI) && f.area * std::fabs(f.T) != 0.)
                faceEmit[i].push_back((int)k);
        }
    }
    for (int q = 0; q < npairs; ++q) {
        const orc_pair& p = pr[q];
        if (p.sdom1 < 0 || p.sdom1 >= ns || p.sdom2 < 0 || p.sdom2 >= ns || p.face1 < 0 ||
            p.face1 >= (int)D->sd[p.sdom1].f.size() || p.face2 < 0 || p.face2 >= (int)D->sd[p.sdom2].f.size()) {
            delete D;
            return nullptr;
        }
        Face& f1 = D->sd[p.sdom1].f[p.face1];
        Face& f2 = D->sd[p.sdom2].f[p.face2];
        if (p.kind == ORC_PERI) {
            // montecarlo/boundary.cpp:524-550
            M3 R; for (int i = 0; i < 9; ++i) R.m[i] = p.rot[i];
            V3 t = mk(p.transl[0], p.transl[1], p.transl[2]);
            double T1 = f1.T, T2 = f2.T;
            f1.T = T1 - T2; f2.T = T2 - T1;
            f1.prot = R; f2.prot = transpose(R);
            f1.ptransl = t;
            V3 mt = mul(transpose(R), t);
            f2.ptransl = mk(-mt[0], -mt[1], -mt[2]);
            f1.pairS = p.sdom2; f1.pairF = p.face2;
            f2.pairS = p.sdom1; f2.pairF = p.face1;
        } else {
            // montecarlo/boundary.cpp:361-369
            f1.inter.push_back(std::make_pair(p.sdom2, p.face2));
            f2.inter.push_back(std::make_pair(p.sdom1, p.face1));
        }
    }
    // montecarlo/domain.cpp:88-102: volume emitter, then face emitters
    long cols = 0;
    for (int i = 0; i < ns; ++i) {
        Sdom& sd = D->sd[i];
        if (sd.emitWeight() != 0.) D->em.push_back(Emitter{i, -1});
        for (int k : faceEmit[i]) D->em.push_back(Emitter{i, k});
        // montecarlo/field.cpp:93-113
        long sp = sd.shape[0] * sd.shape[1] * sd.shape[2];
        if (sp == 0) continue;
        sd.colbeg = cols;
        cols += sp;
    }
    D->cols = cols;
    return D;
}

orc_domain* orc_domain_create(const orc_pped* s, int ns, const orc_pair* pr, int npairs) {
    std::vector<orc_sdom> v(ns > 0 ? ns : 0);
    for (int i = 0; i < ns; ++i) {
        orc_sdom& d = v[i];
        std::memset(&d, 0, sizeof(d));
        d.shape = ORC_PARALLELEPIPED;
        d.ncols = 3;
        for (int k = 0; k < 3; ++k) { d.o[k] = s[i].o[k]; d.div[k] = s[i].div[k]; d.gradT[k] = s[i].gradT[k]; }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) d.mat[3 * c + r] = s[i].M[3 * r + c];
        for (int k = 0; k < 6; ++k) { d.kind[k] = s[i].kind[k]; d.T[k] = s[i].T[k]; }
    }
    return orc_domain_create_shapes(v.data(), ns, pr, npairs);
}

void orc_domain_cell_volumes(const orc_domain* d, double* out) {
    for (const Sdom& s : d->sd) {
        if (s.colbeg < 0) continue;
        long idx[3];
        for (idx[2] = 0; idx[2] < s.shape[2]; ++idx[2])
            for (idx[1] = 0; idx[1] < s.shape[1]; ++idx[1])
                for (idx[0] = 0; idx[0] < s.shape[0]; ++idx[0])
                    out[s.colbeg + flatIndex(s, idx)] = cellVolume(s, idx);
    }
}

double orc_domain_sdom_volume(const orc_domain* d, int s) { return d->sd[s].vol; }

long orc_domain_emitters(const orc_domain* d, double* weights, int* sdom, int* face) {
    for (size_t i = 0; i < d->em.size(); ++i) {
        if (weights) weights[i] = d->emitWeight(d->em[i]);
        if (sdom) sdom[i] = d->em[i].sdom;
        if (face) face[i] = d->em[i].face;
    }
    return (long)d->em.size();
}

void orc_domain_draw_positions(const orc_domain* d, long e, uint64_t seed, long n, double* out) {
    const Emitter& E = d->em[e];
    const Sdom& S = d->sd[E.sdom];
    for (long i = 0; i < n; ++i) {
        Source g;
        g.kind = ORC_RNG_PHILOX;
        g.key[0] = (uint32_t)seed; g.key[1] = (uint32_t)(seed >> 32);
        g.id = (uint32_t)i;
        g.setEvent(0);
        g.word(); g.word();  // drawFluxProp
        V3 x = E.face >= 0 ? drawFacePos(S.f[E.face], g) : drawVolumePos(S, g);
        for (int k = 0; k < 3; ++k) out[3 * i + k] = x[k];
    }
}

int orc_domain_is_inside(const orc_domain* d, int s, const double* x) {
    return d->isInside(s, mk(x[0], x[1], x[2])) ? 1 : 0;
}

void orc_domain_free(orc_domain* d) { delete d; }
long orc_domain_cols(const orc_domain* d) { return d->cols; }

// montecarlo/domain.cpp:188-199 (FilmDomain: PeriP, Diff, Spec)
orc_domain* orc_domain_film(double Lx, double Ly, double Lz, long divy, double dT) {
    orc_pped p;
    std::memset(&p, 0, sizeof(p));
    p.M[0] = Lx; p.M[4] = Ly; p.M[8] = Lz;
    p.div[1] = divy;
    p.gradT[0] = -dT / Lx;
    int k[6] = {ORC_PERI, ORC_DIFF, ORC_SPEC, ORC_PERI, ORC_DIFF, ORC_SPEC};
    for (int i = 0; i < 6; ++i) p.kind[i] = k[i];
    orc_pair q;
    std::memset(&q, 0, sizeof(q));
    q.kind = ORC_PERI; q.sdom1 = 0; q.face1 = 0; q.sdom2 = 0; q.face2 = 3;
    q.transl[0] = Lx;
    q.rot[0] = q.rot[4] = q.rot[8] = 1.;
    return orc_domain_create(&p, 1, &q, 1);
}

// montecarlo/domain.cpp:137-148 (BulkDomain: PeriP, Spec, Spec)
orc_domain* orc_domain_bulk(double L, long divx, double dT) {
    orc_pped p;
    std::memset(&p, 0, sizeof(p));
    p.M[0] = L; p.M[4] = L; p.M[8] = L;
    p.div[0] = divx;
    p.gradT[0] = -dT / L;
    int k[6] = {ORC_PERI, ORC_SPEC, ORC_SPEC, ORC_PERI, ORC_SPEC, ORC_SPEC};
    for (int i = 0; i < 6; ++i) p.kind[i] = k[i];
    orc_pair q;
    std::memset(&q, 0, sizeof(q));
    q.kind = ORC_PERI; q.sdom1 = 0; q.face1 = 0; q.sdom2 = 0; q.face2 = 3;
    q.transl[0] = L;
    q.rot[0] = q.rot[4] = q.rot[8] = 1.;
    return orc_domain_create(&p, 1, &q, 1);
}

void orc_accumulate(const orc_domain* d, int sdom, const double* bpos,
                    const double* epos, const double* amount, long rows,
                    double* data) {
    Field F;
    F.rows = rows; F.cols = d->cols;
    F.data.assign(data, data + rows * d->cols);
    accumulate(*d, sdom, mk(bpos[0], bpos[1], bpos[2]), mk(epos[0], epos[1], epos[2]), amount, F);
    std::memcpy(data, F.data.data(), sizeof(double) * rows * d->cols);
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox(ctr, key, out);
}

uint32_t orc_mt19937_nth(uint32_t seed, long n) {
    std::mt19937 g(seed);
    uint32_t x = 0;
    for (long i = 0; i < n; ++i) x = (uint32_t)g();
    return x;
}

void orc_draw_iso(uint32_t x1, uint32_t x2, double out[3]) {
    uint32_t w[2] = {x1, x2};
    int64_t off[2] = {0, 2};
    Source g; g.kind = ORC_RNG_REPLAY; g.rw = w; g.rpos = off[0]; g.rend = off[1];
    V3 v = drawIso(g);
    for (int i = 0; i < 3; ++i) out[i] = v[i];
}

void orc_draw_aniso(uint32_t x1, uint32_t x2, int bidir, double out[3]) {
    uint32_t w[2] = {x1, x2};
    Source g; g.kind = ORC_RNG_REPLAY; g.rw = w; g.rpos = 0; g.rend = 2;
    V3 v = drawAniso(g, bidir != 0);
    for (int i = 0; i < 3; ++i) out[i] = v[i];
}

void orc_rot_z_to(const double n[3], double R[9]) {
    M3 r = rotZTo(mk(n[0], n[1], n[2]));
    for (int i = 0; i < 9; ++i) R[i] = r.m[i];
}

// montecarlo/problem.cpp:315-342 (constructor) and 370-445 (solve)
int orc_solve(const orc_material* mp, const orc_domain* dp,
              const orc_problem* P, double* out, orc_stats* stats) {
    const orc_material& m = *mp;
    const orc_domain& D = *dp;
    auto t0 = std::chrono::steady_clock::now();
    long nemitter = (long)D.em.size();
    if (nemitter == 0) return -1;
    std::vector<double> weight(nemitter);
    double wsum = 0.;
    for (long i = 0; i < nemitter; ++i) { weight[i] = D.emitWeight(D.em[i]); wsum += weight[i]; }
    std::vector<long> emitCdf(nemitter);
    long nemit = 0;
    for (long i = 0; i < nemitter; ++i) {
        double frac = weight[i] / wsum;
        double rounded = std::ceil(frac * P->nemit - 0.5);
        long n = std::max(1L, (long)rounded);
        nemit += n;
        emitCdf[i] = nemit;
    }
    long maxscat = P->maxscat;
    long maxloop = P->maxloop != 0 ? P->maxloop : 100 * maxscat;
    double power = wsum / nemit * m.fluxSum / 4.;
    // CumTemp / CumFlux (montecarlo/problem.cpp:553-648): size + 1 bins of
    // the scatter count before a flight, step = ceil((maxscat - 1) / size)
    const bool cum = P->problem == ORC_CUMTEMP || P->problem == ORC_CUMFLUX;
    if (P->problem < ORC_TEMP || P->problem > ORC_CUMFLUX) return -1;
    if (cum && (P->cum_size < 1 || maxscat < 2)) return -1;
    const long cumStep = cum ? (maxscat - 1 + P->cum_size - 1) / P->cum_size : 1;
    long rows = P->problem == ORC_TEMP ? 1 : (P->problem == ORC_FLUX ? 3 : (P->problem == ORC_MULTI ? 4 : 0));
    if (P->problem == ORC_CUMTEMP) rows = P->cum_size + 1;
    if (P->problem == ORC_CUMFLUX) rows = 3 * (P->cum_size + 1);
    long cols = D.cols;
    double H = P->horizon;
    bool useH = H > 0.;
    double dt = P->dt;

    int nthreads = P->nthreads > 0 ? P->nthreads : 1;
#ifdef _OPENMP
    if (P->nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    int nchunk = P->rng == ORC_RNG_MT_THREADS ? std::max(1, P->nchunk) : 0;
    // work units: MT chunks (static split as libgomp does) or phonon blocks
    long unitSize = 256;
    long nunits = P->rng == ORC_RNG_MT_THREADS ? nchunk : (nemit + unitSize - 1) / unitSize;
    std::vector<Local> locals(nthreads);
    for (auto& L : locals) {
        L.F.rows = rows; L.F.cols = cols; L.F.data.assign(rows * cols, 0.);
        std::memset(&L.st, 0, sizeof(L.st));
    }
    uint32_t key[2] = {(uint32_t)P->seed, (uint32_t)(P->seed >> 32)};

#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (long u = 0; u < nunits; ++u) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        Local& L = locals[tid];
        long nb, ne;
        std::mt19937 mt;
        if (P->rng == ORC_RNG_MT_THREADS) {
            long q = nemit / nchunk, r = nemit % nchunk;
            if (u < r) { nb = (q + 1) * u; ne = nb + q + 1; }
            else { nb = q * u + r; ne = nb + q; }
            mt.seed((uint32_t)(P->seed + (uint64_t)u));
        } else {
            nb = u * unitSize; ne = std::min(nemit, nb + unitSize);
        }
        for (long n = nb; n < ne; ++n) {
            Source g;
            g.kind = P->rng;
            g.mt = &mt;
            g.key[0] = key[0]; g.key[1] = key[1];
            g.id = (uint32_t)n;
            g.setEvent(0);
            if (P->rng == ORC_RNG_REPLAY) {
                g.rw = P->replay_words; g.rpos = P->replay_offsets[n]; g.rend = P->replay_offsets[n + 1];
            }
            if (P->record_words && P->record_counts) {
                g.rec = P->record_words + n * P->record_cap; g.reccap = P->record_cap;
            }
            double* lg = nullptr;
            long nlog = 0;
            if (P->log && P->log_counts && n < P->log_phonons) lg = P->log + n * P->log_cap * 12;

            long ei = std::upper_bound(emitCdf.begin(), emitCdf.end(), n) - emitCdf.begin();
            const Emitter& E = D.em[ei];
            int si = E.sdom;
            const Sdom* S = &D.sd[si];
            Phonon ph;
            // drawFluxProp (montecarlo/material.cpp:277-280)
            {
                double u1 = g.u01(), u2 = g.u01();
                m.flux.draw(u1, u2, ph.w, ph.p);
            }
            // Emitter::emit (montecarlo/boundary.cpp:378-385)
            V3 pos, dir;
            bool sign;
            if (E.face >= 0) {
                const Face& f = S->f[E.face];
                pos = drawFacePos(f, g);
                dir = mul(f.rot, drawAniso(g, false));
                sign = f.T >= 0.;
            } else {
                pos = drawVolumePos(*S, g);
                dir = mul(S->rot, drawAniso(g, true));
                sign = dot(dir, S->gradT) < 0.;
            }
            ph.sign = sign ? 1 : -1;
            ph.pos = pos;
            ph.dir = normalized(dir);
            drawScatNext(m, ph, g);

            std::vector<double> amountV((size_t)rows, 0.);
            double* amount = amountV.data();
            for (long i = 0; i < maxloop; ++i) {
                g.setEvent((uint32_t)(i + 1));
                Phonon pre = ph;
                double vel = m.velOf(ph.w, ph.p);
                // Subdomain::advect (montecarlo/subdomain.cpp:161-192)
                double minD = ph.scatNext;
                int hit = -1;
                for (int k = 0; k < (int)S->f.size(); ++k) {
                    const Face& f = S->f[k];
                    double nd = dot(f.n, ph.dir);
                    if (nd >= 0.) continue;
                    double dist = -(f.off + dot(f.n, ph.pos)) / nd;
                    if (dist < minD) { minD = dist; hit = k; }
                }
                bool hstop = false;
                if (useH && ph.time + minD / vel > H) {
                    // horizon: fly only up to H, no event
                    minD = (H - ph.time) * vel;
                    hit = -2;
                    hstop = true;
                }
                move(ph, minD, vel);
                if (hstop) ph.time = H;
                bool esc = false;
                if (!hstop) {
                    bool negDist = minD < -S->eps;
                    bool outside = !D.isInside(si, ph.pos);
                    if (negDist || outside) esc = true;
                }
                if (esc) {
                    ph.alive = false;
                    L.st.escapes++;
                    if (lg && nlog < P->log_cap) {
                        double* r = lg + nlog * 12;
                        long ix[3]; coord2index(*S, coordOf(*S, ph.pos), ix);
                        double rec[12] = {(double)i, (double)si, -3., (double)si, (double)flatIndex(*S, ix),
                                          ph.pos[0], ph.pos[1], ph.pos[2], ph.time, (double)ph.nscat,
                                          (double)ph.w, (double)ph.p};
                        std::memcpy(r, rec, sizeof(rec));
                        ++nlog;
                    }
                    break;
                }
                // accumAmt (montecarlo/problem.cpp:473-544) times sign
                double dtm = ph.time - pre.time;
                V3 dx = sub(ph.pos, pre.pos);
                if (P->problem == ORC_TEMP) { amount[0] = ph.sign * dtm; }
                else if (P->problem == ORC_FLUX) { for (int q = 0; q < 3; ++q) amount[q] = ph.sign * dx[q]; }
                else if (P->problem == ORC_MULTI) {
                    amount[0] = ph.sign * dtm;
                    for (int q = 0; q < 3; ++q) amount[q + 1] = ph.sign * dx[q];
                } else {
                    // the bin of the scatter count before the flight
                    // (montecarlo/problem.cpp:589-596,626-633)
                    std::fill(amountV.begin(), amountV.end(), 0.);
                    const long bin = ((long)pre.nscat + cumStep - 1) / cumStep;
                    if (P->problem == ORC_CUMTEMP) amount[bin] = ph.sign * dtm;
                    else for (int q = 0; q < 3; ++q) amount[3 * bin + q] = ph.sign * dx[q];
                }
                accumulate(D, si, pre.pos, ph.pos, amount, L.F);
                V3 endPos = ph.pos;
                int siBefore = si;
                const Sdom* Sb = S;
                if (hstop) {
                    L.st.horizon_stops++;
                } else if (hit >= 0) {
                    const Face& f = S->f[hit];
                    switch (f.kind) {
                    case ORC_SPEC:  // montecarlo/boundary.cpp:283-287
                        ph.dir = normalized(mul(f.refl, ph.dir));
                        break;
                    case ORC_DIFF:  // montecarlo/boundary.cpp:308-312
                        ph.dir = normalized(mul(f.rot, drawAniso(g, false)));
                        ph.nscat++;
                        break;
                    case ORC_ISOT:  // montecarlo/boundary.cpp:455-460
                        ph.alive = false;
                        L.st.absorbed++;
                        break;
                    case ORC_PERI:  // montecarlo/boundary.cpp:516-522
                        ph.pos = add(mul(f.prot, ph.pos), f.ptransl);
                        ph.dir = normalized(mul(f.prot, ph.dir));
                        si = f.pairS;
                        break;
                    case ORC_INTER: {  // montecarlo/boundary.cpp:349-359
                        int to = -1;
                        if (f.inter.size() == 1) to = f.inter[0].first;
                        else
                            for (auto& pr2 : f.inter)
                                if (D.isInside(pr2.first, ph.pos)) { to = pr2.first; break; }
                        if (to < 0) { ph.alive = false; L.st.escapes++; }
                        else si = to;
                        break;
                    }
                    }
                    S = &D.sd[si];
                } else {
                    // Material::scatter (montecarlo/material.cpp:298-303)
                    double u1 = g.u01(), u2 = g.u01();
                    m.scat.draw(u1, u2, ph.w, ph.p);
                    ph.dir = normalized(drawIso(g));
                    ph.nscat++;
                    drawScatNext(m, ph, g);
                    L.st.scatters++;
                }
                if (!hstop) L.st.events++;
                if (lg && nlog < P->log_cap) {
                    double* r = lg + nlog * 12;
                    long ix[3]; coord2index(*Sb, coordOf(*Sb, endPos), ix);
                    double rec[12] = {(double)i, (double)siBefore, (double)(hstop ? -2 : hit), (double)si,
                                      (double)flatIndex(*Sb, ix), endPos[0], endPos[1], endPos[2], ph.time,
                                      (double)ph.nscat, (double)ph.w, (double)ph.p};
                    std::memcpy(r, rec, sizeof(rec));
                    ++nlog;
                }
                if (g.exhausted) break;
                if (hstop || !ph.alive) break;
                if (ph.nscat >= maxscat) { L.st.maxscat_stops++; break; }
            }
            if (g.exhausted) L.st.replay_exhausted++;
            if (dt > 0.) L.st.phonon_steps += std::max(1.0, std::ceil(ph.time / dt));
            if (lg) P->log_counts[n] = nlog;
            if (g.rec) P->record_counts[n] = g.reccount;
        }
    }

    // reduction (montecarlo/main.cpp:162-165), postProc and cell volume
    std::vector<double> sum(rows * cols, 0.);
    orc_stats st;
    std::memset(&st, 0, sizeof(st));
    for (auto& L : locals) {
        for (long i = 0; i < rows * cols; ++i) sum[i] += L.F.data[i];
        st.phonon_steps += L.st.phonon_steps;
        st.events += L.st.events; st.scatters += L.st.scatters; st.escapes += L.st.escapes;
        st.horizon_stops += L.st.horizon_stops; st.maxscat_stops += L.st.maxscat_stops;
        st.absorbed += L.st.absorbed; st.replay_exhausted += L.st.replay_exhausted;
    }
    // CumTemp / CumFlux postProc: cumulative sums over the bins
    // (montecarlo/problem.cpp:598-606,636-645)
    if (cum) {
        const long per = P->problem == ORC_CUMTEMP ? 1 : 3;
        for (long c = 0; c < cols; ++c)
            for (long r = per; r < rows; ++r) sum[c * rows + r] += sum[c * rows + r - per];
    }
    // montecarlo/problem.cpp:439-444
    for (int si = 0; si < (int)D.sd.size(); ++si) {
        const Sdom& s = D.sd[si];
        if (s.colbeg < 0) continue;
        long sp = s.shape[0] * s.shape[1] * s.shape[2];
        std::vector<double> cvs((size_t)sp);
        {
            long idx[3];
            for (idx[2] = 0; idx[2] < s.shape[2]; ++idx[2])
                for (idx[1] = 0; idx[1] < s.shape[1]; ++idx[1])
                    for (idx[0] = 0; idx[0] < s.shape[0]; ++idx[0]) cvs[flatIndex(s, idx)] = cellVolume(s, idx);
        }
        for (long c = s.colbeg; c < s.colbeg + sp; ++c)
            for (long r = 0; r < rows; ++r) {
                const double cv = cvs[c - s.colbeg];
                double v = sum[c * rows + r];
                if (P->problem == ORC_TEMP || P->problem == ORC_CUMTEMP || (P->problem == ORC_MULTI && r == 0))
                    v = v / m.energySum;
                out[c * rows + r] = power * (v / cv);
            }
    }
    st.nemit = nemit;
    st.power = power;
    st.rows = rows;
    st.cols = cols;
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    st.threads = nthreads;
    if (stats) *stats = st;
    return 0;
}

}  // extern "C"
