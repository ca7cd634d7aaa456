// mc_api.cu -- host side of the C ABI declared in include/mc_gb300.h.
//
// Builds, in FP64 on the host, everything the kernels read: the material's
// velocity / relaxation tables and integer inverse-CDF thresholds
// (montecarlo/material.cpp:51-75,154-234), the subdomains' reduced-coordinate
// geometry, face normals, rotations and pair maps
// (montecarlo/subdomain.cpp:41-71, montecarlo/boundary.cpp:28-37,44-56,
// 361-369,524-550), the emitter list and phonon allocation
// (montecarlo/domain.cpp:88-102, montecarlo/problem.cpp:315-342), and
// post-processes the FP64 tallies (montecarlo/problem.cpp:439-551).

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <string>
#include <vector>

#include "../../include/mc_gb300.h"
#include "mc_launch.h"
#include "mc_matbuild.h"

using namespace mcg;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cudaFail(cudaError_t e, const char* where) {
    return fail(MC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                                    \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cudaFail(e_, #call);          \
    } while (0)

const double HBAR = 1.054560652927e-034;  // montecarlo/constants.h:18
const double KB = 1.380648e-023;          // montecarlo/constants.h:19
const double DMIN = std::numeric_limits<double>::min();
const double DEPS = std::numeric_limits<double>::epsilon();

int ensureDevice() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(MC_ERR_NO_DEVICE, "no CUDA device: the GB300 kernels cannot run (no CPU fallback)");
    return MC_OK;
}

// ---------------------------------------------------------------- vectors
struct V3 { double v[3]; double& operator[](int i) { return v[i]; } double operator[](int i) const { return v[i]; } };
V3 mk(double a, double b, double c) { V3 r; r[0] = a; r[1] = b; r[2] = c; return r; }
double dot(const V3& a, const V3& b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
V3 cross(const V3& a, const V3& b) {
    return mk(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
V3 unit(const V3& a) {
    double z = dot(a, a);
    if (!(z > 0.)) return a;
    double s = std::sqrt(z);
    return mk(a[0] / s, a[1] / s, a[2] / s);
}
struct M3 { double m[9]; };
M3 eye() { M3 r{}; r.m[0] = r.m[4] = r.m[8] = 1.; return r; }
M3 mmul(const M3& a, const M3& b) {
    M3 r{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = (a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j]) + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}
V3 mvec(const M3& a, const V3& x) {
    return mk((a.m[0] * x[0] + a.m[1] * x[1]) + a.m[2] * x[2], (a.m[3] * x[0] + a.m[4] * x[1]) + a.m[5] * x[2],
              (a.m[6] * x[0] + a.m[7] * x[1]) + a.m[8] * x[2]);
}
M3 transp(const M3& a) { M3 r{}; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[3 * i + j] = a.m[3 * j + i]; return r; }
double det3(const M3& a) {
    const double* m = a.m;
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}
M3 inv3(const M3& a) {
    const double* m = a.m;
    double d = det3(a);
    M3 r{};
    r.m[0] = (m[4] * m[8] - m[5] * m[7]) / d; r.m[1] = (m[2] * m[7] - m[1] * m[8]) / d; r.m[2] = (m[1] * m[5] - m[2] * m[4]) / d;
    r.m[3] = (m[5] * m[6] - m[3] * m[8]) / d; r.m[4] = (m[0] * m[8] - m[2] * m[6]) / d; r.m[5] = (m[2] * m[3] - m[0] * m[5]) / d;
    r.m[6] = (m[3] * m[7] - m[4] * m[6]) / d; r.m[7] = (m[1] * m[6] - m[0] * m[7]) / d; r.m[8] = (m[0] * m[4] - m[1] * m[3]) / d;
    return r;
}
V3 colOf(const M3& a, int c) { return mk(a.m[c], a.m[3 + c], a.m[6 + c]); }

// Rotation taking z-hat to n: half-angle quaternion about z x n, as a
// matrix; for n = -z the rotation by pi about x.
M3 rotZTo(const V3& nIn) {
    V3 v1 = unit(nIn);
    double c = v1[2];
    double qw, qx, qy, qz;
    if (c < -1. + 1e-12) {
        qw = 0.; qx = 1.; qy = 0.; qz = 0.;
    } else {
        V3 axis = cross(mk(0., 0., 1.), v1);
        double s = std::sqrt((1. + c) * 2.);
        double invs = 1. / s;
        qx = axis[0] * invs; qy = axis[1] * invs; qz = axis[2] * invs;
        qw = s * 0.5;
    }
    double tx = 2. * qx, ty = 2. * qy, tz = 2. * qz;
    double twx = tx * qw, twy = ty * qw, twz = tz * qw;
    double txx = tx * qx, txy = ty * qx, txz = tz * qx;
    double tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
    M3 r{};
    r.m[0] = 1. - (tyy + tzz); r.m[1] = txy - twz; r.m[2] = txz + twy;
    r.m[3] = txy + twz; r.m[4] = 1. - (txx + tzz); r.m[5] = tyz - twx;
    r.m[6] = txz - twy; r.m[7] = tyz + twx; r.m[8] = 1. - (txx + tyy);
    return r;
}

// Two-level discrete distribution (montecarlo/material.cpp:123-147) as
// integer inverse-CDF thresholds (cdfThreshold): the bins by their
// running sum over the bins' totals, the branches of a bin by theirs.
void buildThresholds(const std::vector<double>& pdf, long nw, long np, std::vector<unsigned long long>& wthr,
                     std::vector<unsigned long long>& pthr) {
    std::vector<double> rowSum(nw);
    pthr.assign(nw * np, 4294967296ull);
    for (long w = 0; w < nw; ++w) rowSum[w] = branchThresholds(pdf.data(), w, np, pthr.data());
    double acc = 0.;
    for (long w = 0; w < nw; ++w) acc += rowSum[w];
    wthr.resize(nw);
    double pre = 0.;
    for (long w = 0; w < nw; ++w) {
        pre += rowSum[w];
        wthr[w] = cdfThreshold(pre / acc);
    }
}

template <typename R>
struct DevTables {
    R* vel = nullptr;
    R* vt = nullptr;
    unsigned long long *wthr = nullptr, *pthr = nullptr, *fwthr = nullptr, *fpthr = nullptr;
};

}  // namespace

struct mc_material_s {
    long nw = 0, np = 0;
    double T = 0.;
    std::vector<double> omega, vel, tau;
    double energySum = 0., fluxSum = 0., scatSum = 0., cond = 0.;
    std::vector<unsigned long long> swthr, spthr, fwthr, fpthr;
};

namespace {

int buildMaterial(const double* disp, long nw, long np, const double* relax, double T, mc_material_s** out) {
    if (!disp || !relax || nw <= 0 || np <= 0 || np > 255 || nw > 65535)
        return fail(MC_ERR_ARG, "Invalid dispersion file");
    if (!(T > 0.)) return fail(MC_ERR_ARG, "temperature must be positive");
    mc_material_s* m = new mc_material_s;
    m->nw = nw; m->np = np; m->T = T;
    m->omega.resize(nw);
    m->vel.resize(nw * np);
    m->tau.assign(nw * np, 0.);
    std::vector<double> domega(nw), dos(nw * np);
    const long nc = 2 + 2 * np;
    for (long w = 0; w < nw; ++w) {
        m->omega[w] = disp[w * nc];
        domega[w] = disp[w * nc + 1];
        for (long p = 0; p < np; ++p) {
            m->vel[w * np + p] = disp[w * nc + 2 + 2 * p];
            dos[w * np + p] = disp[w * nc + 3 + 2 * p];
        }
    }
    for (long p = 0; p < np; ++p)
        for (int j = 0; j < 2; ++j)
            if (relax[p * 8 + 4 * j] < 0.) { delete m; return fail(MC_ERR_ARG, "Scattering times cannot be negative"); }
    // the temperature-dependent tables with the host/device formulas of
    // mc_matbuild.h (the device build of many temperatures gives the same bits)
    for (long w = 0; w < nw; ++w)
        for (long p = 0; p < np; ++p) m->tau[w * np + p] = 1. / tauInverse(relax, p, m->omega[w], T);
    for (long i = 0; i < nw * np; ++i)
        if (!std::isfinite(m->tau[i])) { delete m; return fail(MC_ERR_ARG, "Scattering time model produced infinite values"); }
    for (long i = 0; i < nw * np; ++i)
        if (!(m->vel[i] > DMIN)) { delete m; return fail(MC_ERR_ARG, "Velocity must be nonzero"); }
    std::vector<double> epdf(nw * np), fpdf(nw * np), spdf(nw * np);
    double es = 0., fs = 0., ss = 0., k = 0.;
    for (long w = 0; w < nw; ++w) {
        const double dedT = dEdT(m->omega[w], T);
        for (long p = 0; p < np; ++p) {
            long i = w * np + p;
            epdf[i] = dedT * dos[i] * domega[w];
            fpdf[i] = m->vel[i] * epdf[i];
            spdf[i] = epdf[i] / m->tau[i];
            es += epdf[i]; fs += fpdf[i]; ss += spdf[i];
            k += m->tau[i] * (m->vel[i] * m->vel[i]) * epdf[i];
        }
    }
    if (!(fs > 0.) || !(ss > 0.)) { delete m; return fail(MC_ERR_ARG, "material has no phonons to draw"); }
    m->energySum = es; m->fluxSum = fs; m->scatSum = ss; m->cond = k / 3.;
    buildThresholds(spdf, nw, np, m->swthr, m->spthr);
    buildThresholds(fpdf, nw, np, m->fwthr, m->fpthr);
    *out = m;
    return MC_OK;
}

bool readAll(const char* path, std::vector<double>& v) {
    std::ifstream f(path);
    if (!f) return false;
    double x;
    while (f >> x) v.push_back(x);
    return true;
}

struct HostFace {
    int kind;
    int shape = 0;            // 0 Parallelogram, 1 Triangle, 2 Polygon
    V3 n, o, si, sj;          // inward normal, origin, shape vectors
    std::vector<V3> verts;    // Polygon: vertices relative to o
    std::vector<double> tri;  // Polygon: triangle areas
    double area, T;
    int pairS = -1, pairF = -1;
    M3 R = eye();
    V3 t = mk(0, 0, 0);
    std::vector<std::pair<int, int>> inter;  // Inter pairs (subdomain, face) in makePair order
};

V3 addv(const V3& a, const V3& b) { return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
V3 subv(const V3& a, const V3& b) { return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
V3 sclv(double s, const V3& a) { return mk(s * a[0], s * a[1], s * a[2]); }

// Boundary(o, shape) with the shape's normal and area: Parallelogram
// (montecarlo/boundary.cpp:121-152), Triangle (154-186), Polygon<N>
// (188-258; triangles (v_n, v_n+1) for n < N - 2).
HostFace makeFace(int kind, double T, const V3& o, int shape, const V3& si, const V3& sj,
                  const std::vector<V3>& verts = std::vector<V3>()) {
    HostFace F;
    F.kind = kind; F.T = T; F.o = o; F.shape = shape; F.si = si; F.sj = sj;
    if (shape == 2) {
        F.verts = verts;
        double a = 0.;
        for (size_t k = 0; k + 1 < verts.size(); ++k) {
            V3 cr = cross(verts[k], verts[k + 1]);
            F.tri.push_back(std::sqrt(dot(cr, cr)) / 2.);
            a += F.tri.back();
        }
        F.area = a;
        F.n = unit(cross(verts[0], verts[1]));
    } else {
        V3 cr = cross(si, sj);
        F.n = unit(cr);
        F.area = std::sqrt(dot(cr, cr)) / (shape == 1 ? 2. : 1.);
    }
    return F;
}

// A subdomain on the host: the reference's Subdomain matrix (for the
// escape tolerance and the cell coordinates), the shape's volume and
// faces, and the device frame (a box holding the shape) with its walk grid.
struct HostSdom {
    int shape = MC_PARALLELEPIPED;
    V3 o;
    M3 M;                 // Subdomain::matrix (matBase for Prism / Pyramid)
    long div[3];          // Subdomain divisions
    double vol = 0.;
    std::vector<HostFace> f;
    std::vector<V3> col;  // the constructor's matrix columns
    std::vector<double> subvol;  // Prism / Pyramid: volume(mat)
    V3 fo;                // frame origin and matrix
    M3 FM;
    double edge = 0.;     // longest matrix column
};

// Faces of each shape in bdry<I>() order and its volume: Parallelepiped
// (montecarlo/subdomain.h:145-158), TriangularPrism (224-236),
// Tetrahedron (303-314), Prism<N> (386-410, InitSidesF 458-475, PrismImpl
// montecarlo/subdomain.cpp:376-397) and Pyramid<N> (subdomain.h:524-547,
// InitSidesF 595-613, PyramidImpl subdomain.cpp:409-431).
int buildShape(const mc_sdom_desc& p, HostSdom& H) {
    const int N = p.ncols;
    H.shape = p.shape;
    H.o = mk(p.o[0], p.o[1], p.o[2]);
    H.col.resize(N);
    for (int i = 0; i < N; ++i) H.col[i] = mk(p.mat[3 * i], p.mat[3 * i + 1], p.mat[3 * i + 2]);
    const std::vector<V3>& c = H.col;
    const V3& o = H.o;
    auto K = [&](int i) { return p.kind[i]; };
    auto T = [&](int i) { return p.T[i]; };
    if (p.shape == MC_PARALLELEPIPED || p.shape == MC_TRIANGULAR_PRISM || p.shape == MC_TETRAHEDRON) {
        if (N != 3) return fail(MC_ERR_ARG, "this shape takes a 3-column matrix");
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) H.M.m[3 * r + q] = c[q][r];
        for (int k = 0; k < 3; ++k) H.div[k] = p.div[k];
        const double d = det3(H.M);
        if (p.shape == MC_PARALLELEPIPED) {
            H.vol = d;
            V3 fo[6] = {o, o, o, addv(o, c[0]), addv(o, c[1]), addv(o, c[2])};
            V3 fi[6] = {c[1], c[2], c[0], c[2], c[0], c[1]};
            V3 fj[6] = {c[2], c[0], c[1], c[1], c[2], c[0]};
            for (int k = 0; k < 6; ++k) H.f.push_back(makeFace(K(k), T(k), fo[k], 0, fi[k], fj[k]));
        } else if (p.shape == MC_TRIANGULAR_PRISM) {
            H.vol = d / 2.;
            H.f.push_back(makeFace(K(0), T(0), o, 0, c[1], c[2]));
            H.f.push_back(makeFace(K(1), T(1), o, 0, c[2], c[0]));
            H.f.push_back(makeFace(K(2), T(2), o, 1, c[0], c[1]));
            H.f.push_back(makeFace(K(3), T(3), addv(o, c[0]), 0, c[2], subv(c[1], c[0])));
            H.f.push_back(makeFace(K(4), T(4), addv(o, c[2]), 1, c[1], c[0]));
        } else {
            H.vol = d / 6.;
            H.f.push_back(makeFace(K(0), T(0), o, 1, c[1], c[2]));
            H.f.push_back(makeFace(K(1), T(1), o, 1, c[2], c[0]));
            H.f.push_back(makeFace(K(2), T(2), o, 1, c[0], c[1]));
            H.f.push_back(makeFace(K(3), T(3), addv(o, c[0]), 1, subv(c[2], c[0]), subv(c[1], c[0])));
        }
    } else if (p.shape == MC_PRISM || p.shape == MC_PYRAMID) {
        if (N < 4 || N > MC_MAX_SDOM_COLS) return fail(MC_ERR_ARG, "Prism / Pyramid take 4 to 9 columns");
        const bool prism = p.shape == MC_PRISM;
        for (int r = 0; r < 3; ++r) { H.M.m[3 * r] = c[1][r]; H.M.m[3 * r + 1] = c[N - 1][r]; H.M.m[3 * r + 2] = c[0][r]; }
        const long d1 = p.div[0] < 0 ? -1 : 0;
        H.div[0] = H.div[1] = H.div[2] = d1;
        // volume(mat): col(i) x col(i+1) . col(0) for i < N - 2 (as the
        // reference computes it), / 2 (Prism) or / 6 (Pyramid)
        double vs = 0.;
        for (int i = 0; i < N - 2; ++i) {
            H.subvol.push_back(dot(cross(c[i], c[i + 1]), c[0]) / (prism ? 2. : 6.));
            vs += H.subvol.back();
        }
        H.vol = vs;
        std::vector<V3> bot(c.begin() + 1, c.end());
        H.f.push_back(makeFace(K(0), T(0), o, 2, mk(0, 0, 0), mk(0, 0, 0), bot));
        int base = 1;
        if (prism) {
            std::vector<V3> top(bot.rbegin(), bot.rend());
            H.f.push_back(makeFace(K(1), T(1), addv(o, c[0]), 2, mk(0, 0, 0), mk(0, 0, 0), top));
            base = 2;
        }
        for (int ind = 0; ind < N; ++ind) {
            V3 pp = ind != 0 ? c[ind] : mk(0, 0, 0);
            V3 i = prism ? c[0] : (ind != 0 ? subv(c[0], c[ind]) : c[0]);
            V3 j = sclv(-1., pp);
            if (ind != N - 1) j = addv(j, c[ind + 1]);
            H.f.push_back(makeFace(K(base + ind), T(base + ind), addv(o, pp), prism ? 0 : 1, i, j));
        }
    } else {
        return fail(MC_ERR_ARG, "invalid subdomain shape");
    }
    if (!(H.vol >= DMIN)) return fail(MC_ERR_ARG, "Volume too small, check vector order");
    for (const V3& x : H.col) H.edge = std::max(H.edge, std::sqrt(dot(x, x)));
    for (const HostFace& F : H.f) {
        if (F.kind < MC_SPEC || F.kind > MC_INTER) return fail(MC_ERR_ARG, "invalid face kind");
        if ((F.kind == MC_SPEC || F.kind == MC_DIFF || F.kind == MC_INTER) && F.T != 0.)
            return fail(MC_ERR_ARG, "Cannot specify temperature");
    }
    // device frame: the shape's own unit cell, except for Prism / Pyramid
    // (a one-cell field): the box around the vertices in the matBase basis
    H.fo = o;
    H.FM = H.M;
    if (p.shape == MC_PRISM || p.shape == MC_PYRAMID) {
        M3 Mi = inv3(H.M);
        double lo[3] = {0., 0., 0.}, hi[3] = {0., 0., 0.};
        std::vector<V3> pts;
        pts.push_back(mk(0, 0, 0));
        for (int i = 1; i < N; ++i) pts.push_back(c[i]);
        const size_t nb = pts.size();
        if (p.shape == MC_PRISM)
            for (size_t i = 0; i < nb; ++i) pts.push_back(addv(pts[i], c[0]));
        else
            pts.push_back(c[0]);
        for (const V3& q : pts) {
            V3 l = mvec(Mi, q);
            for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], l[k]); hi[k] = std::max(hi[k], l[k]); }
        }
        H.fo = addv(o, mvec(H.M, mk(lo[0], lo[1], lo[2])));
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) H.FM.m[3 * r + q] = H.M.m[3 * r + q] * (hi[q] - lo[q]);
    }
    return MC_OK;
}

// Subdomain::cellVol (ParallelepipedImpl montecarlo/subdomain.cpp:269-273,
// TriangularPrismImpl 283-307, TetrahedronImpl 321-346, PrismImpl and
// PyramidImpl 394-397,428-431), as the reference computes them.
double cellVolume(const HostSdom& H, const long sh[3], const long idx[3]) {
    const double sp = (double)(sh[0] * sh[1] * sh[2]);
    if (H.shape == MC_PARALLELEPIPED) return H.vol / sp;
    if (H.shape == MC_PRISM || H.shape == MC_PYRAMID) return H.vol;
    const int dim = H.shape == MC_TRIANGULAR_PRISM ? 2 : 3;
    double f0 = 1.;
    for (int k = 0; k < dim; ++k) f0 -= (double)idx[k] / (double)sh[k];
    if (f0 <= 0.) return 0.;
    double f1 = f0;
    for (int k = 0; k < dim; ++k) f1 -= 1. / (double)sh[k];
    if (f1 >= 0.) return H.vol / sp;
    if (dim == 2) {
        double frac = std::pow(f0, 2);
        for (int i = 0; i < 2; ++i) {
            double f = f0 - 1. / (double)sh[i];
            if (f > 0.) frac += -1. * std::pow(f, 2);
        }
        return H.vol * frac / (2. * (double)sh[2]);
    }
    static const int pts[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}};
    double frac = std::pow(f0, 3);
    for (int i = 0; i < 6; ++i) {
        const int sum = pts[i][0] + pts[i][1] + pts[i][2];
        double f = f0;
        for (int k = 0; k < 3; ++k) f -= (double)pts[i][k] / (double)sh[k];
        if (f > 0.) frac += ((sum % 2) ? -1. : 1.) * std::pow(f, 3);
    }
    return H.vol * frac / 6.;
}

// Emission pieces of a non-Parallelepiped emitter in the subdomain's frame
// coordinates u = diag(S) FM^-1 (x - fo): u = U0 + L c for the folded
// uniforms c of Emitter::drawPos (TriangularPrismImpl / TetrahedronImpl
// montecarlo/subdomain.cpp:309-373, Prism / Pyramid volDist 399-441,
// Triangle / Polygon<N> montecarlo/boundary.cpp:180-186,246-256).
void setPiece(EmitterD& E, int k, const HostSdom& H, const double S[3], const V3& origin, const V3& e0,
              const V3& e1, const V3& e2) {
    M3 Fi = inv3(H.FM);
    V3 u0 = mvec(Fi, subv(origin, H.fo));
    V3 ev[3] = {mvec(Fi, e0), mvec(Fi, e1), mvec(Fi, e2)};
    for (int r = 0; r < 3; ++r) {
        E.U0[k][r] = S[r] * u0[r];
        for (int q = 0; q < 3; ++q) E.L[k][3 * r + q] = S[r] * ev[q][r];
    }
}
void setThresholds(EmitterD& E, const std::vector<double>& w) {
    double acc = 0.;
    for (double x : w) acc += x;
    double pre = 0.;
    for (size_t i = 0; i < w.size(); ++i) { pre += w[i]; E.thr[i] = cdfThreshold(pre / acc); }
}

}  // namespace

struct mc_domain_s {
    std::vector<mc_sdom_desc> desc;
    std::vector<int> slot;                // device slot of each subdomain
    std::vector<int> refOfSlot;           // subdomain of each slot (-1: a continuation)
    bool needGen = false;                 // other shapes, continuations or several Inter pairs
    std::vector<EmitterD> em;
    std::vector<double> emWeight;
    std::vector<long> colbeg;
    long cols = 0;
    std::vector<double> cellVol;
    std::vector<SdomD<double>> sd;        // FP64 device image
};

namespace {

int buildDomain(const mc_sdom_desc* ps, int n, const mc_pair_desc* qs, int nq, mc_domain_s** out) {
    if (!ps || n <= 0) return fail(MC_ERR_ARG, "Domain setup not complete");
    if (n > MAX_SDOM) return fail(MC_ERR_UNSUPPORTED, "more than 64 subdomains");
    std::unique_ptr<mc_domain_s> D(new mc_domain_s);
    D->desc.assign(ps, ps + n);
    D->sd.resize(n);
    std::vector<HostSdom> H(n);
    std::vector<std::vector<int>> faceEmit(n);
    for (int s = 0; s < n; ++s) {
        if (int rc = buildShape(ps[s], H[s])) return rc;
        for (int k = 0; k < 3; ++k)
            if (H[s].div[k] >= MAX_SHAPE) return fail(MC_ERR_UNSUPPORTED, "more than 511 cells along an axis");
        // construction registers the emitting faces whose weight is nonzero
        // (montecarlo/subdomain.cpp:205-212)
        for (size_t f = 0; f < H[s].f.size(); ++f) {
            const HostFace& F = H[s].f[f];
            if ((F.kind == MC_ISOT || F.kind == MC_PERI) && F.area * std::fabs(F.T) != 0.) faceEmit[s].push_back((int)f);
        }
    }
    for (int q = 0; q < nq; ++q) {
        const mc_pair_desc& P = qs[q];
        if (P.sdom1 < 0 || P.sdom1 >= n || P.sdom2 < 0 || P.sdom2 >= n || P.face1 < 0 ||
            P.face1 >= (int)H[P.sdom1].f.size() || P.face2 < 0 || P.face2 >= (int)H[P.sdom2].f.size())
            return fail(MC_ERR_ARG, "pair index out of range");
        HostFace& a = H[P.sdom1].f[P.face1];
        HostFace& b = H[P.sdom2].f[P.face2];
        if (a.kind != P.kind || b.kind != P.kind) return fail(MC_ERR_ARG, "pair kind does not match faces");
        // the makePair checks (montecarlo/boundary.cpp:363-368,527-535):
        // unit normals within 1e-12, plane offsets within 1e-9 of the
        // larger subdomain edge
        const double L = std::max(H[P.sdom1].edge, H[P.sdom2].edge);
        auto near = [](const V3& x, const V3& y) { return std::sqrt(dot(subv(x, y), subv(x, y))) <= 1e-12; };
        if (P.kind == MC_PERI) {
            if (a.pairS >= 0 || b.pairS >= 0) return fail(MC_ERR_ARG, "Boundary already paired");
            M3 R; std::memcpy(R.m, P.rot, sizeof(R.m));
            V3 t = mk(P.transl[0], P.transl[1], P.transl[2]);
            M3 RRt = mmul(R, transp(R));
            for (int i = 0; i < 9; ++i)
                if (std::fabs(RRt.m[i] - eye().m[i]) > 1e-12) return fail(MC_ERR_ARG, "Rotation matrix must be orthogonal");
            if (!near(mvec(R, a.n), sclv(-1., b.n))) return fail(MC_ERR_ARG, "Rotation matrix incorrect");
            const V3 tf = addv(sclv(dot(a.n, a.o), mvec(R, a.n)), t);
            if (std::fabs(dot(b.n, tf) - dot(b.n, b.o)) > 1e-9 * L) return fail(MC_ERR_ARG, "Translation vector incorrect");
            double T1 = a.T, T2 = b.T;
            a.T = T1 - T2; b.T = T2 - T1;
            a.R = R; b.R = transp(R);
            a.t = t;
            V3 mt = mvec(transp(R), t);
            b.t = mk(-mt[0], -mt[1], -mt[2]);
            a.pairS = P.sdom2; a.pairF = P.face2;
            b.pairS = P.sdom1; b.pairF = P.face1;
        } else if (P.kind == MC_INTER) {
            if (!near(a.n, sclv(-1., b.n))) return fail(MC_ERR_ARG, "Boundary normals not antiparallel");
            if (std::fabs(dot(a.n, a.o) - dot(a.n, b.o)) > 1e-9 * L) return fail(MC_ERR_ARG, "Boundaries planes not the same");
            a.inter.push_back(std::make_pair(P.sdom2, P.face2));
            b.inter.push_back(std::make_pair(P.sdom1, P.face1));
            if (a.pairS < 0) { a.pairS = P.sdom2; a.pairF = P.face2; }
            if (b.pairS < 0) { b.pairS = P.sdom1; b.pairF = P.face1; }
        } else {
            return fail(MC_ERR_ARG, "pair kind must be Peri or Inter");
        }
    }
    for (int s = 0; s < n; ++s)
        for (const HostFace& F : H[s].f)
            if ((F.kind == MC_PERI || F.kind == MC_INTER) && F.pairS < 0)
                return fail(MC_ERR_ARG, "Domain setup not complete: unpaired face");
    // device slots: a subdomain with more than MAX_FACES faces, or with
    // Inter faces paired more than once, also takes a continuation slot
    std::vector<int> extraFaces(n, 0), cand(n, 0);
    int nslot = 0;
    D->slot.resize(n);
    for (int s = 0; s < n; ++s) {
        extraFaces[s] = std::max(0, (int)H[s].f.size() - MAX_FACES);
        for (const HostFace& F : H[s].f)
            if (F.inter.size() > 1) cand[s] += (int)F.inter.size();
        if (extraFaces[s] + cand[s] > MAX_FACES)
            return fail(MC_ERR_UNSUPPORTED, "too many faces and Inter pairs for one subdomain");
        D->slot[s] = nslot;
        D->refOfSlot.push_back(s);
        ++nslot;
        if (extraFaces[s] + cand[s] > 0) { D->refOfSlot.push_back(-1); ++nslot; }
        if (H[s].shape != MC_PARALLELEPIPED || extraFaces[s] + cand[s] > 0) D->needGen = true;
    }
    if (nslot > MAX_SDOM) return fail(MC_ERR_UNSUPPORTED, "more than 64 subdomain slots");
    D->sd.assign(nslot, SdomD<double>());
    for (SdomD<double>& x : D->sd) {
        std::memset(&x, 0, sizeof(x));
        x.colbeg = -1;
        x.accum = -2;
    }
    // subdomain images, emitters and columns
    long cols = 0;
    for (int s = 0; s < n; ++s) {
        const mc_sdom_desc& p = ps[s];
        const HostSdom& h = H[s];
        const bool gen = h.shape != MC_PARALLELEPIPED;
        SdomD<double>& S = D->sd[D->slot[s]];
        std::memset(&S, 0, sizeof(S));
        M3 Mi = inv3(h.FM);
        std::memcpy(S.M, h.FM.m, sizeof(S.M));
        std::memcpy(S.Minv, Mi.m, sizeof(Mi.m));
        bool neg = false;
        int npos = 0;
        for (int k = 0; k < 3; ++k) {
            S.o[k] = h.fo[k];
            if (h.div[k] < 0) neg = true;
            if (h.div[k] > 0) ++npos;
            S.gradT[k] = p.gradT[k];
        }
        S.gen = gen ? 1 : 0;
        S.nface = (int)h.f.size();
        // Subdomain::accumFlag (montecarlo/subdomain.cpp:47-70)
        if (neg) S.accum = -2;
        else if (npos == 0) S.accum = -1;
        else if (npos == 1) { int d = 0; for (int k = 1; k < 3; ++k) if (h.div[k] > h.div[d]) d = k; S.accum = d; }
        else S.accum = npos + 1;
        // walk cells: the tally cells, refined to WALK_CELLS on axes without
        // tally cells when the field is 0-D or 1-D
        long tsh[3];
        for (int k = 0; k < 3; ++k) {
            tsh[k] = std::max(h.div[k], 1L);
            const bool virt = neg || (h.div[k] <= 0 && S.accum <= 2);
            S.shape[k] = virt ? WALK_CELLS : (int)tsh[k];
            S.S[k] = S.shape[k];
        }
        S.tstride[0] = (!neg && h.div[0] > 0) ? 1 : 0;
        S.tstride[1] = (!neg && h.div[1] > 0) ? (int)tsh[0] : 0;
        S.tstride[2] = (!neg && h.div[2] > 0) ? (int)(tsh[0] * tsh[1]) : 0;
        M3 gr = rotZTo(unit(mk(p.gradT[0], p.gradT[1], p.gradT[2])));
        std::memcpy(S.grot, gr.m, sizeof(gr.m));
        double maxn = 0.;
        for (int c = 0; c < 3; ++c) { V3 cc = colOf(h.M, c); maxn = std::max(maxn, std::sqrt(dot(cc, cc))); }
        S.eps = 100. * DEPS * maxn;  // FP32 images rescale this
        double gn = std::sqrt(dot(mk(p.gradT[0], p.gradT[1], p.gradT[2]), mk(p.gradT[0], p.gradT[1], p.gradT[2])));
        double vw = 2. * h.vol * gn;  // montecarlo/subdomain.cpp:250-253
        if (vw != 0.) {
            EmitterD E;
            std::memset(&E, 0, sizeof(E));
            E.sdom = D->slot[s]; E.face = -1; E.fold = -1; E.ncoord = 3; E.npiece = 1;
            if (gen) {
                const std::vector<V3>& c = h.col;
                if (h.shape == MC_PRISM || h.shape == MC_PYRAMID) {
                    E.fold = h.shape == MC_PRISM ? FOLD_PRISM : FOLD_TETRA;
                    E.npiece = (int)h.subvol.size();
                    if (E.npiece > MAX_PIECES) return fail(MC_ERR_UNSUPPORTED, "too many sub-volumes");
                    for (int k = 0; k < E.npiece; ++k) setPiece(E, k, h, S.S, h.o, c[k + 1], c[k + 2], c[0]);
                    setThresholds(E, h.subvol);
                } else {
                    E.fold = h.shape == MC_TRIANGULAR_PRISM ? FOLD_PRISM : FOLD_TETRA;
                    setPiece(E, 0, h, S.S, h.o, c[0], c[1], c[2]);
                    E.thr[0] = 4294967296ull;
                }
            }
            D->em.push_back(E);
            D->emWeight.push_back(vw);
        }
        for (int f : faceEmit[s]) {
            const HostFace& F = h.f[f];
            EmitterD E;
            std::memset(&E, 0, sizeof(E));
            E.sdom = D->slot[s]; E.face = f; E.fold = -1; E.ncoord = 2; E.npiece = 1;
            if (gen) {
                const V3 z = mk(0, 0, 0);
                if (F.shape == 2) {
                    E.fold = FOLD_TRIANGLE;
                    E.npiece = (int)F.tri.size();
                    if (E.npiece > MAX_PIECES) return fail(MC_ERR_UNSUPPORTED, "too many polygon vertices");
                    for (int k = 0; k < E.npiece; ++k) setPiece(E, k, h, S.S, F.o, F.verts[k], F.verts[k + 1], z);
                    setThresholds(E, F.tri);
                } else {
                    E.fold = F.shape == 1 ? FOLD_TRIANGLE : FOLD_NONE;
                    setPiece(E, 0, h, S.S, F.o, F.si, F.sj, z);
                    E.thr[0] = 4294967296ull;
                }
            }
            D->em.push_back(E);
            D->emWeight.push_back(F.area * std::fabs(F.T));  // montecarlo/boundary.cpp:413-416
        }
        long sp = neg ? 0 : tsh[0] * tsh[1] * tsh[2];
        if (sp == 0) { S.colbeg = -1; D->colbeg.push_back(-1); continue; }
        S.colbeg = (int)cols;
        D->colbeg.push_back(cols);
        long idx[3];
        for (idx[2] = 0; idx[2] < tsh[2]; ++idx[2])
            for (idx[1] = 0; idx[1] < tsh[1]; ++idx[1])
                for (idx[0] = 0; idx[0] < tsh[0]; ++idx[0]) D->cellVol.push_back(cellVolume(h, tsh, idx));
        cols += sp;
    }
    D->cols = cols;
    // faces: normals, rotations, planes, pair maps in frame coordinates
    auto faceAt = [&](int s, int f) -> FaceD<double>& {
        SdomD<double>* S = &D->sd[D->slot[s]];
        return f < MAX_FACES ? S->f[f] : S[1].f[f - MAX_FACES];
    };
    // pair map of face f of subdomain s into face tf of subdomain ts:
    // u' = diag(S') Minv' (R (o + M diag(1/S) u) + t - o')
    auto setMap = [&](FaceD<double>& G, int s, int f, const M3& R, const V3& tr, int ts, int tf) {
        const SdomD<double>& S = D->sd[D->slot[s]];
        const SdomD<double>& T2 = D->sd[D->slot[ts]];
        G.to = D->slot[ts];
        G.toface = T2.gen ? -1 : tf;
        bool id = true;
        for (int i = 0; i < 9; ++i) if (R.m[i] != eye().m[i]) id = false;
        G.ident = id ? 1 : 0;
        std::memcpy(G.Rd, R.m, sizeof(R.m));
        M3 Mi2; std::memcpy(Mi2.m, T2.Minv, sizeof(Mi2.m));
        M3 M1; std::memcpy(M1.m, S.M, sizeof(M1.m));
        M3 A = mmul(mmul(Mi2, R), M1);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) A.m[3 * i + j] = A.m[3 * i + j] * T2.S[i] / S.S[j];
        V3 Ro = mvec(R, mk(S.o[0], S.o[1], S.o[2]));
        V3 x0 = mk(Ro[0] + tr[0] - T2.o[0], Ro[1] + tr[1] - T2.o[1], Ro[2] + tr[2] - T2.o[2]);
        V3 b = mvec(Mi2, x0);
        std::memcpy(G.A, A.m, sizeof(A.m));
        for (int k = 0; k < 3; ++k) G.b[k] = T2.S[k] * b[k];
        // tangential identity: same axis, A = I and no tangential shift
        // (within rounding of the FP64 products)
        const int ax = f % 3;
        bool tang = !S.gen && !T2.gen && f < 6 && (tf % 3) == ax;
        for (int i = 0; i < 3 && tang; ++i) {
            if (i == ax) continue;  // the normal coordinate is snapped
            for (int j = 0; j < 3; ++j)
                if (std::fabs(A.m[3 * i + j] - (i == j ? 1. : 0.)) > 1e-12) tang = false;
        }
        for (int k = 0; k < 3 && tang; ++k)
            if (k != ax && std::fabs(G.b[k]) > 1e-12 * T2.S[k]) tang = false;
        G.tang = tang ? 1 : 0;
    };
    for (int s = 0; s < n; ++s) {
        SdomD<double>& S = D->sd[D->slot[s]];
        int nextCand = extraFaces[s];
        for (int f = 0; f < S.nface; ++f) {
            const HostFace& F = H[s].f[f];
            FaceD<double>& G = faceAt(s, f);
            G.kind = F.kind;
            G.to = -1; G.toface = -1; G.ident = 1; G.more = 0;
            for (int k = 0; k < 3; ++k) G.n[k] = F.n[k];
            M3 r = rotZTo(F.n);
            std::memcpy(G.rot, r.m, sizeof(r.m));
            M3 I = eye();
            std::memcpy(G.Rd, I.m, sizeof(I.m));
            std::memcpy(G.A, I.m, sizeof(I.m));
            G.T = F.T;
            if (S.gen) {
                // signed distance n.x - n.fo at x = o + M diag(1/S) u
                M3 SM;
                std::memcpy(SM.m, S.M, sizeof(SM.m));
                V3 g = mvec(transp(SM), F.n);
                for (int k = 0; k < 3; ++k) G.gp[k] = g[k] / S.S[k];
                G.gp[3] = dot(F.n, subv(mk(S.o[0], S.o[1], S.o[2]), F.o));
            }
            if (F.kind == MC_PERI) {
                setMap(G, s, f, F.R, F.t, F.pairS, F.pairF);
            } else if (F.kind == MC_INTER && F.inter.size() == 1) {
                setMap(G, s, f, eye(), mk(0, 0, 0), F.pairS, F.pairF);
            } else if (F.kind == MC_INTER) {
                // several pairs: the first whose subdomain holds the position
                // (montecarlo/boundary.cpp:349-359); the candidates go to the
                // continuation slot, each with S_k / height_k of its target
                G.more = ((int)F.inter.size() << 8) | nextCand;
                for (const auto& q : F.inter) {
                    FaceD<double>& C = D->sd[D->slot[s] + 1].f[nextCand++];
                    std::memset(&C, 0, sizeof(C));
                    C.kind = MC_INTER;
                    setMap(C, s, f, eye(), mk(0, 0, 0), q.first, q.second);
                    const HostSdom& th = H[q.first];
                    const SdomD<double>& T2 = D->sd[D->slot[q.first]];
                    const double vol = std::fabs(det3(th.M));
                    for (int k = 0; k < 3; ++k) {
                        V3 cr = cross(colOf(th.M, (k + 1) % 3), colOf(th.M, (k + 2) % 3));
                        C.n[k] = T2.S[k] / (vol / std::sqrt(dot(cr, cr)));
                    }
                }
            }
        }
    }
    *out = D.release();
    return MC_OK;
}

// A Parallelepiped description as a general one (mat column-major).
mc_sdom_desc sdomOfPped(const mc_pped_desc& p) {
    mc_sdom_desc d;
    std::memset(&d, 0, sizeof(d));
    d.shape = MC_PARALLELEPIPED;
    d.ncols = 3;
    for (int k = 0; k < 3; ++k) { d.o[k] = p.o[k]; d.div[k] = p.div[k]; d.gradT[k] = p.gradT[k]; }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) d.mat[3 * c + r] = p.M[3 * r + c];
    for (int k = 0; k < 6; ++k) { d.kind[k] = p.kind[k]; d.T[k] = p.T[k]; }
    return d;
}

// Field rows of a problem (montecarlo/problem.cpp:470-471,502-503,535-536,
// 578-581,615-618): Temp 1, Flux 3, Multi 4, CumTemp size + 1, CumFlux
// 3 (size + 1).
long problemRows(int problem, long size) {
    switch (problem) {
    case MC_TEMP: return 1;
    case MC_FLUX: return 3;
    case MC_MULTI: return 4;
    case MC_CUMTEMP: return size + 1;
    default: return 3 * (size + 1);
    }
}
// CumTemp / CumFlux scatters per bin, ceil((maxscat - 1) / size)
// (montecarlo/problem.cpp:558-564); 1 for the other problems.
int cumStepOf(int problem, long maxscat, long size) {
    if (problem != MC_CUMTEMP && problem != MC_CUMFLUX) return 1;
    return (int)((maxscat - 1 + size - 1) / size);
}
// Whether row class k (see rowClass) holds times rather than displacements.
bool timeClass(int problem, int k) {
    return problem == MC_CUMTEMP || ((problem == MC_TEMP || problem == MC_MULTI) && k == 0);
}
// Problem arguments the kernels need (the reference asserts or divides by
// zero otherwise).
int checkProblem(const mc_problem_desc& p) {
    if (p.problem < MC_TEMP || p.problem > MC_CUMFLUX) return fail(MC_ERR_ARG, "Invalid problem");
    if (p.problem == MC_CUMTEMP || p.problem == MC_CUMFLUX) {
        if (p.cum_size < 1) return fail(MC_ERR_ARG, "cum_size must be >= 1");
        if (p.maxscat < 2 || p.maxscat >= (1L << 31)) return fail(MC_ERR_ARG, "CumTemp / CumFlux need 2 <= maxscat < 2^31");
        if (p.cum_size > (1L << 20)) return fail(MC_ERR_ARG, "cum_size too large");
    }
    return MC_OK;
}
// postProc of the summed raw field, rows x cols column-major, in place
// (montecarlo/problem.cpp:478-481,511-514,546-551,598-606,636-645): the
// cumulative sums over the scatter-count bins, then the division of the
// time rows by the material's energy sum.
void postProcess(int problem, long rows, long cols, double energySum, double* v) {
    if (problem == MC_CUMTEMP || problem == MC_CUMFLUX) {
        const long per = problem == MC_CUMTEMP ? 1 : 3;
        for (long c = 0; c < cols; ++c)
            for (long r = per; r < rows; ++r) v[c * rows + r] += v[c * rows + r - per];
    }
    for (long c = 0; c < cols; ++c)
        for (long r = 0; r < rows; ++r)
            if (problem == MC_TEMP || problem == MC_CUMTEMP || (problem == MC_MULTI && r == 0))
                v[c * rows + r] /= energySum;
}

template <typename R>
void castSdom(const SdomD<double>& a, SdomD<R>& b, bool f32) {
    std::memset(&b, 0, sizeof(b));
    for (int i = 0; i < 9; ++i) { b.Minv[i] = (R)a.Minv[i]; b.M[i] = (R)a.M[i]; b.grot[i] = (R)a.grot[i]; }
    for (int i = 0; i < 3; ++i) {
        b.o[i] = (R)a.o[i]; b.S[i] = (R)a.S[i]; b.gradT[i] = (R)a.gradT[i];
        b.shape[i] = a.shape[i]; b.tstride[i] = a.tstride[i];
    }
    // escape tolerance: 100 ulp of the largest edge in the flight precision
    b.eps = (R)(f32 ? a.eps / DEPS * (double)std::numeric_limits<float>::epsilon() : a.eps);
    b.accum = a.accum;
    b.colbeg = a.colbeg;
    b.gen = a.gen;
    b.nface = a.nface;
    for (int f = 0; f < MAX_FACES; ++f) {
        const FaceD<double>& x = a.f[f];
        FaceD<R>& y = b.f[f];
        y.kind = x.kind; y.to = x.to; y.toface = x.toface; y.ident = x.ident; y.tang = x.tang; y.more = x.more;
        for (int i = 0; i < 3; ++i) { y.n[i] = (R)x.n[i]; y.b[i] = (R)x.b[i]; }
        for (int i = 0; i < 9; ++i) { y.rot[i] = (R)x.rot[i]; y.Rd[i] = (R)x.Rd[i]; y.A[i] = (R)x.A[i]; }
        for (int i = 0; i < 4; ++i) y.gp[i] = (R)x.gp[i];
        y.T = (R)x.T;
    }
}

}  // namespace

// ================================================================ session
struct mc_session_s {
    mc_material_h mat = nullptr;
    mc_domain_h dom = nullptr;
    mc_problem_desc desc{};
    int prec = 32;
    bool replay = false, logging = false;
    bool dyn = false;
    int sinceCompact = 0;
    int tm = TM_SHARED;
    int block = 256, grid = 0;
    size_t smem = 0;
    long nemit = 0;
    double power = 0.;
    long maxloop = 0;
    int rows = 1;
    int step = 0;         // next window start
    int launches = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timing = false;
    // device buffers
    void* state = nullptr;       // two halves
    bool pooled = false;         // buffers from the stream-ordered pool (freed on the stream)
    size_t stateBytes = 0;
    void* tables = nullptr;
    void* dom_d = nullptr;
    EmitterD* em_d = nullptr;
    long long* cdf_d = nullptr;
    unsigned long long* cnt_d = nullptr;   // counters + 2 live slots
    unsigned int* status_d = nullptr;
    double* tally_d = nullptr;
    double* csum_d = nullptr;
    uint32_t* rwords_d = nullptr;
    long long* roff_d = nullptr;
    uint32_t* rcur_d = nullptr;
    double* log_d = nullptr;
    int* logcnt_d = nullptr;
    int lean = -1;                // static schedule: axis of the lean flight, or -1
    bool gen = false;             // the domain has subdomains other than the Parallelepiped
    long long slots = 0;          // phonon slots per half of the state
    unsigned* reg_d = nullptr;    // static schedule: front / back live counts
                                  // per block region, one array per half
    int parity = 0;               // which half holds the live phonons
    double vmax = 0.;             // largest group velocity of the material
    Params<float> p32{};
    Params<double> p64{};
};

// The device's default stream-ordered memory pool keeps freed memory for
// reuse by this process instead of returning it at each synchronisation (a
// process setting, not a device one).
static void keepPooledMemory() {
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    });
}

// A session's device buffers come from the pool on the session's stream
// (stream != null), so that creating and destroying sessions costs neither
// driver allocations nor the device-wide synchronisation of cudaFree;
// batches and servers keep plain allocations (stream == null).
#ifndef MC_SESSION_POOL
#define MC_SESSION_POOL 1
#endif
// whether the current device has stream-ordered memory pools (else
// sessions allocate with cudaMalloc)
static bool poolsSupported() {
    int dev = 0, ok = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&ok, cudaDevAttrMemoryPoolsSupported, dev) != cudaSuccess) return false;
    return ok != 0;
}
static cudaError_t devAlloc(void** p, size_t bytes, cudaStream_t pool) {
    if (pool) {
        keepPooledMemory();
        return cudaMallocAsync(p, bytes, pool);
    }
    return cudaMalloc(p, bytes);
}
// host to device, in stream order on the pool's stream (from pageable
// memory the call returns once the host buffer has been staged)
static cudaError_t devUpload(void* dst, const void* src, size_t bytes, cudaStream_t pool) {
    if (pool) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, pool);
    return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
}

namespace {

// Material tables in the flight precision, thresholds, guide table: one
// device allocation; fills the table pointers of P.
template <typename R>
int uploadMaterial(const mc_material_s& m, void** buf, Params<R>& P, double& vmax, cudaStream_t pool = nullptr) {
    const size_t nt = (size_t)m.nw * m.np;
    size_t tb = 2 * sizeof(R) * nt + sizeof(unsigned long long) * (2 * m.nw + 2 * nt) + 2 * GUIDE + 128;
    CK(devAlloc(buf, tb, pool));
    char* base = (char*)*buf;
    std::vector<R> vel(nt), vt(nt);
    for (size_t i = 0; i < nt; ++i) { vel[i] = (R)m.vel[i]; vt[i] = (R)(m.vel[i] * m.tau[i]); }
    vmax = 0.;
    for (size_t i = 0; i < nt; ++i) vmax = std::max(vmax, m.vel[i]);
    // every table 16-byte aligned (the kernels stage them by bulk copies)
    auto al16 = [](char* b) { return (char*)(((uintptr_t)b + 15) & ~(uintptr_t)15); };
    P.vel = (R*)base; base += sizeof(R) * nt;
    base = al16(base);
    P.vt = (R*)base; base += sizeof(R) * nt;
    base = al16(base);
    P.wthr = (unsigned long long*)base; base += 8 * m.nw;
    P.pthr = (unsigned long long*)base; base += 8 * nt;
    P.fwthr = (unsigned long long*)base; base += 8 * m.nw;
    P.fpthr = (unsigned long long*)base; base += 8 * nt;
    base = al16(base);
    P.wguide = (const uint16_t*)base; base += 2 * GUIDE;
    CK(devUpload((void*)P.vel, vel.data(), sizeof(R) * nt, pool));
    CK(devUpload((void*)P.vt, vt.data(), sizeof(R) * nt, pool));
    CK(devUpload((void*)P.wthr, m.swthr.data(), 8 * m.nw, pool));
    CK(devUpload((void*)P.pthr, m.spthr.data(), 8 * nt, pool));
    CK(devUpload((void*)P.fwthr, m.fwthr.data(), 8 * m.nw, pool));
    CK(devUpload((void*)P.fpthr, m.fpthr.data(), 8 * nt, pool));
    {
        // guide table: first bin whose threshold exceeds k * 2^32 / GUIDE
        std::vector<uint16_t> g(GUIDE);
        for (int k = 0; k < GUIDE; ++k) {
            const unsigned long long x = (unsigned long long)k << (32 - GUIDE_BITS);
            long i = 0;
            while (i < m.nw - 1 && x >= m.swthr[i]) ++i;
            g[k] = (uint16_t)i;
        }
        CK(devUpload((void*)P.wguide, g.data(), 2 * GUIDE, pool));
    }
    P.nw = (int)m.nw;
    P.np = (int)m.np;
    return MC_OK;
}

// Subdomain images, emitters and the phonon allocation of a requested
// count (montecarlo/problem.cpp:315-342); fills P.sd / em / emitCdf.
template <typename R>
int uploadDomain(const mc_domain_s& D, double fluxSum, long nemitReq, void** sd_d, EmitterD** em_d,
                 long long** cdf_d, Params<R>& P, long& nemit, double& power, cudaStream_t pool = nullptr) {
    std::vector<SdomD<R>> sd(D.sd.size());
    for (size_t i = 0; i < sd.size(); ++i) castSdom(D.sd[i], sd[i], sizeof(R) == 4);
    CK(devAlloc(sd_d, sizeof(SdomD<R>) * sd.size(), pool));
    CK(devUpload(*sd_d, sd.data(), sizeof(SdomD<R>) * sd.size(), pool));
    P.sd = (const SdomD<R>*)*sd_d;
    P.nsd = (int)sd.size();
    const long ne = (long)D.em.size();
    if (ne == 0) return fail(MC_ERR_ARG, "No phonons to emit");
    double wsum = 0.;
    for (double w : D.emWeight) wsum += w;
    std::vector<long long> cdf(ne);
    long long tot = 0;
    for (long i = 0; i < ne; ++i) {
        double frac = D.emWeight[i] / wsum;
        double rounded = std::ceil(frac * nemitReq - 0.5);
        tot += std::max(1LL, (long long)rounded);
        cdf[i] = tot;
    }
    nemit = (long)tot;
    power = wsum / (double)tot * fluxSum / 4.;
    for (long i = 0; i < ne; ++i)
        if (!(D.emWeight[i] > 0.)) return fail(MC_ERR_ARG, "No phonons to emit");
    CK(devAlloc((void**)em_d, sizeof(EmitterD) * ne, pool));
    CK(devUpload(*em_d, D.em.data(), sizeof(EmitterD) * ne, pool));
    CK(devAlloc((void**)cdf_d, sizeof(long long) * ne, pool));
    CK(devUpload(*cdf_d, cdf.data(), sizeof(long long) * ne, pool));
    P.em = *em_d;
    P.emitCdf = *cdf_d;
    P.nem = (int)ne;
    return MC_OK;
}

template <typename R>
int setupSession(mc_session_s* S) {
    const mc_material_s& m = *S->mat;
    const mc_domain_s& D = *S->dom;
    Params<R> P{};
    cudaStream_t pool = (MC_SESSION_POOL && poolsSupported()) ? S->stream : nullptr;
    S->pooled = pool != nullptr;
    int rc = uploadMaterial<R>(m, &S->tables, P, S->vmax, pool);
    if (rc) return rc;
    rc = uploadDomain<R>(D, m.fluxSum, S->desc.nemit, &S->dom_d, &S->em_d, &S->cdf_d, P, S->nemit, S->power, pool);
    if (rc) return rc;
    // counters: C_NCOUNTERS + two (front, back) live-count pairs + the
    // dynamic launches' slot counter
    CK(devAlloc((void**)&S->cnt_d, sizeof(unsigned long long) * (C_NCOUNTERS + 5), pool));
    CK(devAlloc((void**)&S->status_d, sizeof(unsigned int), pool));
    S->rows = (int)problemRows(S->desc.problem, S->desc.cum_size);
    CK(devAlloc((void**)&S->tally_d, sizeof(double) * (size_t)S->rows * std::max(D.cols, 1L), pool));
    P.problem = S->desc.problem; P.rows = S->rows; P.cols = (int)D.cols;
    P.cumStep = cumStepOf(S->desc.problem, S->desc.maxscat, S->desc.cum_size);
    P.nemit = S->nemit;
    P.maxscat = S->desc.maxscat;
    P.maxloop = S->maxloop;
    P.dt = (R)S->desc.dt;
    P.nsteps = (int)S->desc.nsteps;
    P.ksteps = S->desc.steps_per_launch;
    P.key0 = (uint32_t)S->desc.seed;
    P.key1 = (uint32_t)(S->desc.seed >> 32);
    P.counters = S->cnt_d;
    P.qglobal = MC_DYN_GLOBAL_QUEUE ? S->cnt_d + C_NCOUNTERS + 4 : nullptr;
    P.cap = (unsigned long long)S->nemit;
    P.status = S->status_d;
    P.tally = S->tally_d;
    CK(devAlloc((void**)&S->csum_d, sizeof(double) * 4, pool));
    P.csum = S->csum_d;
    // replay
    if (S->replay) {
        const int64_t* off = S->desc.replay_offsets;
        long long nw = off[S->nemit];
        if (off[0] != 0 || nw < 0) return fail(MC_ERR_ARG, "replay offsets must start at 0");
        for (long i = 0; i < S->nemit; ++i)
            if (off[i + 1] < off[i]) return fail(MC_ERR_ARG, "replay offsets must not decrease");
        CK(devAlloc((void**)&S->rwords_d, sizeof(uint32_t) * std::max(nw, 1LL), pool));
        if (nw) CK(devUpload(S->rwords_d, S->desc.replay_words, sizeof(uint32_t) * nw, pool));
        CK(devAlloc((void**)&S->roff_d, sizeof(long long) * (S->nemit + 1), pool));
        CK(devUpload(S->roff_d, off, sizeof(long long) * (S->nemit + 1), pool));
        CK(devAlloc((void**)&S->rcur_d, sizeof(uint32_t) * S->nemit, pool));
        P.rwords = S->rwords_d; P.roff = S->roff_d; P.rcur = S->rcur_d;
    }
    if (S->logging) {
        long long ln = std::min<long long>(S->desc.log_phonons, S->nemit);
        CK(devAlloc((void**)&S->log_d, sizeof(double) * 12 * (size_t)ln * S->desc.log_cap + 8, pool));
        CK(devAlloc((void**)&S->logcnt_d, sizeof(int) * (size_t)std::max(ln, 1LL), pool));
        P.log = S->log_d; P.logcap = S->desc.log_cap; P.logn = ln; P.logcount = S->logcnt_d;
    }
    // launch configuration
    const size_t tallyB = smemTallyBytes(S->rows, (int)D.cols);
    S->tm = S->desc.tally_mode;
    if (S->tm == MC_TALLY_AUTO) S->tm = tallyB <= 32 * 1024 ? TM_SHARED : TM_GLOBAL;
    const int maxBlock = S->dyn ? 256 : staticConsumers<R>();
    S->block = S->desc.block_size > 0 ? S->desc.block_size : maxBlock;
    if (S->block % 32 || S->block > maxBlock)
        return fail(MC_ERR_ARG, S->dyn || sizeof(R) == 8 ? "block_size must be a multiple of 32, <= 256"
                                                         : "block_size must be a multiple of 32, <= 768");
    // static schedule with a shared 1-D field along one axis in every
    // subdomain (and no replay or log): the kernel with the lean flight
    S->lean = -1;
    S->gen = D.needGen;
    if (!S->dyn && !S->replay && !S->logging && S->tm == TM_SHARED) {
        const int k = D.sd[0].accum;
        bool same = k >= 0 && k <= 2;
        for (const auto& x : D.sd) same = same && x.accum == k && !D.needGen;
        if (same) S->lean = k;
    }
    // FP32 lean flights tally into a carry-free copy of the field (exact
    // while a block runs at most SPLIT_MAX_FLIGHTS of them per launch,
    // checked below)
    const bool split = S->lean >= 0 && sizeof(R) == 4;
    P.tabGlobal = (!S->dyn && MC_STATIC_TABLES_GLOBAL) ? 1 : 0;
    {
        const SmemLayout L = singleLayout<R>((int)m.nw, (int)m.np, (int)D.sd.size(), S->rows, (int)D.cols,
                                             S->tm == TM_SHARED, split, !P.tabGlobal);
        S->smem = L.total;
        setSingleLayout(P, L);
        // static schedule: the state stages after the tables
        if (!S->dyn) S->smem = staticStageOffset(L.total) + STATIC_STAGES * staticStageBytes<R>(S->block);
    }
    if (S->smem > 227 * 1024) return fail(MC_ERR_UNSUPPORTED, "shared-memory tables exceed 227 KB");
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int occ = S->lean >= 0 ? advanceLeanOccupancy<R>(S->lean, S->block, S->smem)
                           : advanceOccupancy<R>(S->dyn, S->replay, S->logging, S->tm, S->gen, S->block, S->smem);
    if (occ <= 0) return fail(MC_ERR_UNSUPPORTED, "advance kernel cannot launch with this configuration");
    S->grid = S->desc.grid_blocks > 0 ? S->desc.grid_blocks : occ * nsm;
    if (split && S->desc.grid_blocks == 0 && (S->nemit + S->grid - 1) / S->grid > SPLIT_MAX_FLIGHTS) {
        // whole waves of resident blocks rather than more phonons per block
        // than the carry-free copy holds (a partial last wave would run its
        // few blocks alone)
        const long long need = (S->nemit + SPLIT_MAX_FLIGHTS - 1) / SPLIT_MAX_FLIGHTS;
        const long long wave = (long long)occ * nsm;
        S->grid = (int)((need + wave - 1) / wave * wave);
    }
    if (split && (S->nemit + S->grid - 1) / S->grid > SPLIT_MAX_FLIGHTS) {
        // too many phonons per block of a requested grid for the carry-free
        // copy: the walker for every phonon
        S->lean = -1;
        P.smSplit = 0;
        occ = advanceOccupancy<R>(S->dyn, S->replay, S->logging, S->tm, S->gen, S->block, S->smem);
        if (occ <= 0) return fail(MC_ERR_UNSUPPORTED, "advance kernel cannot launch with this configuration");
        S->grid = S->desc.grid_blocks > 0 ? S->desc.grid_blocks : occ * nsm;
    }
    // state: two halves of (P0, P1, P2). The static schedule cuts each half
    // into one region of C slots per block of its (fixed) grid.
    size_t n = (size_t)S->nemit;
    if (!S->dyn) {
        const long long C = (S->nemit + S->grid - 1) / S->grid;
        n = (size_t)C * (size_t)S->grid;
        CK(devAlloc((void**)&S->reg_d, sizeof(unsigned) * 4 * (size_t)S->grid, pool));
        P.regCap = C;
    }
    using V4 = typename Vec4<R>::T;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t half = 2 * al(sizeof(V4) * n) + al(sizeof(uint4) * n);
    S->stateBytes = 2 * (sizeof(V4) * 2 + sizeof(uint4)) * n;
    S->slots = (long long)n;
    CK(devAlloc(&S->state, 2 * half, pool));
    char* sb = (char*)S->state;
    V4* h0[2]; V4* h1[2]; uint4* h2[2];
    for (int h = 0; h < 2; ++h) {
        h0[h] = (V4*)sb; sb += al(sizeof(V4) * n);
        h1[h] = (V4*)sb; sb += al(sizeof(V4) * n);
        h2[h] = (uint4*)sb; sb += al(sizeof(uint4) * n);
    }
    // halves
    Params<R>* dst = nullptr;
    if (sizeof(R) == 4) dst = (Params<R>*)&S->p32; else dst = (Params<R>*)&S->p64;
    *dst = P;
    struct Halves { V4* a[2]; V4* b[2]; uint4* c[2]; };
    static_assert(sizeof(void*) == 8, "64-bit");
    dst->P0in = h0[0]; dst->P1in = h1[0]; dst->P2in = h2[0];
    dst->P0out = h0[1]; dst->P1out = h1[1]; dst->P2out = h2[1];
    return MC_OK;
}

template <typename R>
Params<R>& paramsOf(mc_session_s* S);
template <> Params<float>& paramsOf<float>(mc_session_s* S) { return S->p32; }
template <> Params<double>& paramsOf<double>(mc_session_s* S) { return S->p64; }

template <typename R>
int emitT(mc_session_s* S) {
    Params<R>& P = paramsOf<R>(S);
    // emission writes the first half
    using V4 = typename Vec4<R>::T;
    V4* a0 = P.P0in; V4* a1 = P.P1in; uint4* a2 = P.P2in;
    if (S->parity == 1) { a0 = P.P0out; a1 = P.P1out; a2 = P.P2out; }
    Params<R> E = P;
    E.P0out = a0; E.P1out = a1; E.P2out = a2;
    CK(cudaMemsetAsync(S->cnt_d, 0, sizeof(unsigned long long) * (C_NCOUNTERS + 4), S->stream));
    CK(cudaMemsetAsync(S->status_d, 0, sizeof(unsigned int), S->stream));
    CK(cudaMemsetAsync(S->csum_d, 0, sizeof(double) * 4, S->stream));
    CK(cudaMemsetAsync(S->tally_d, 0, sizeof(double) * (size_t)S->rows * std::max(S->dom->cols, 1L), S->stream));
    if (S->replay) CK(cudaMemsetAsync(S->rcur_d, 0, sizeof(uint32_t) * S->nemit, S->stream));
    if (S->logging) {
        CK(cudaMemsetAsync(S->logcnt_d, 0, sizeof(int) * std::min<long long>(S->desc.log_phonons, S->nemit), S->stream));
        CK(cudaMemsetAsync(S->log_d, 0xFF, sizeof(double) * 12 * (size_t)std::min<long long>(S->desc.log_phonons, S->nemit) * S->desc.log_cap, S->stream));
    }
    if (!S->dyn) {
        // region counts of the emitted half (the kernel sets the fronts)
        E.regIn = S->reg_d + 2 * (size_t)S->grid * S->parity;
        CK(cudaMemsetAsync(E.regIn, 0, sizeof(unsigned) * 2 * (size_t)S->grid, S->stream));
    }
    // live counts of the emitted half: all in front
    unsigned long long n = (unsigned long long)S->nemit;
    CK(cudaMemcpyAsync(S->cnt_d + C_NCOUNTERS + 2 * S->parity, &n, sizeof(n), cudaMemcpyHostToDevice, S->stream));
    CK(launchEmit<R>(E, S->replay, S->stream));
    CK(cudaStreamSynchronize(S->stream));  // n lives on the host stack
    S->step = 0;
    S->launches = 1;
    return MC_OK;
}

// Fixed-point quantum of the tallies for one row. `flight` bounds what one
// phonon adds in a window (the window itself for time rows, vmax x window
// for displacement rows). FP32 flight: 2^-27 of it, so that every flight's
// amount converts to a 32-bit integer with room for the lean flights'
// carry-free field (2^18 flights per block); a block's sums (at most
// `perBlock` phonons x 2^27) stay inside int64. The quantum is 7.5e-9 of
// the largest flight, below the FP32 flight's own rounding. FP64 flight:
// 2^-61 of perBlock x flight, converted to 64 bits.
double tallyQuantum(bool f32, double flight, double perBlock) {
    return f32 ? std::ldexp(flight * 1.0001, -27) : std::ldexp(perBlock * flight * 1.0001, -61);
}

template <typename R>
void setQuanta(const mc_session_s* S, Params<R>& P) {
    const int keff = (int)std::min<long>(S->desc.steps_per_launch, S->desc.nsteps - S->step);
    const double window = (double)keff * S->desc.dt;
    const double perBlock = std::ceil((double)S->nemit / ((double)S->grid * S->block)) * S->block;
    for (int r = 0; r < 4; ++r) {
        const double q = tallyQuantum(sizeof(R) == 4, window * (timeClass(S->desc.problem, r) ? 1.0 : S->vmax), perBlock);
        P.tq[r] = q;
        P.tqinv[r] = (R)(1.0 / q);
    }
}

template <typename R>
int advanceT(mc_session_s* S, int nl, int* done) {
    Params<R>& P0 = paramsOf<R>(S);
    const int nsteps = (int)S->desc.nsteps;
    for (int l = 0; l < nl && S->step < nsteps; ++l) {
        Params<R> P = P0;
        if (S->parity == 1) {
            std::swap(P.P0in, P.P0out); std::swap(P.P1in, P.P1out); std::swap(P.P2in, P.P2out);
        }
        P.step0 = S->step;
        setWindow(P);
        setQuanta(S, P);
        unsigned long long* cur = S->cnt_d + C_NCOUNTERS + 2 * S->parity;
        unsigned long long* oth = S->cnt_d + C_NCOUNTERS + 2 * (S->parity ^ 1);
        if (S->dyn) {
            // in place: slots [0, cur[0]) of the current half, survivors
            // counted in cur[1]
            P.P0out = P.P0in; P.P1out = P.P1in; P.P2out = P.P2in;
            P.live_in = cur;
            P.live_out = cur + 1;
            CK(cudaMemsetAsync(cur + 1, 0, sizeof(unsigned long long), S->stream));
            // one launch-wide slot counter only for long windows: a claim
            // per refilled lane is then rare enough for one address
            if (P.wKeff < MC_DYN_QUEUE_MIN_STEPS) P.qglobal = nullptr;
            if (P.qglobal) CK(cudaMemsetAsync(P.qglobal, 0, sizeof(unsigned long long), S->stream));
            CK(launchAdvance<R>(P, true, S->replay, S->logging, S->tm, S->gen, S->grid, S->block, S->smem,
                                S->stream));
            S->launches++;
            S->step += S->desc.steps_per_launch;
            if (S->desc.compact_interval > 0 && ++S->sinceCompact >= S->desc.compact_interval &&
                S->step < nsteps) {
                Params<R> Q = P0;
                if (S->parity == 1) {
                    std::swap(Q.P0in, Q.P0out); std::swap(Q.P1in, Q.P1out); std::swap(Q.P2in, Q.P2out);
                }
                Q.live_in = cur;
                Q.live_out = oth;
                CK(cudaMemsetAsync(oth, 0, 2 * sizeof(unsigned long long), S->stream));
                CK(launchCompact<R>(Q, S->grid, S->stream));
                S->launches++;
                S->parity ^= 1;
                S->sinceCompact = 0;
            }
        } else {
            // block regions of the current half -> the other half
            P.regIn = S->reg_d + 2 * (size_t)S->grid * S->parity;
            P.regOut = S->reg_d + 2 * (size_t)S->grid * (S->parity ^ 1);
            if (S->lean >= 0) CK(launchAdvanceLean<R>(P, S->lean, S->grid, S->block, S->smem, S->stream));
            else CK(launchAdvance<R>(P, false, S->replay, S->logging, S->tm, S->gen, S->grid, S->block, S->smem,
                                     S->stream));
            S->parity ^= 1;
            S->step += S->desc.steps_per_launch;
            S->launches++;
        }
    }
    if (done) *done = S->step >= nsteps ? 1 : 0;
    return MC_OK;
}

int resultImpl(mc_session_s* S, double* out, mc_stats* st) {
    CK(cudaStreamSynchronize(S->stream));
    const mc_domain_s& D = *S->dom;
    const mc_material_s& m = *S->mat;
    std::vector<unsigned long long> c(C_NCOUNTERS + 4);
    unsigned int status = 0;
    CK(cudaMemcpy(c.data(), S->cnt_d, sizeof(unsigned long long) * c.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&status, S->status_d, sizeof(status), cudaMemcpyDeviceToHost));
    const size_t nval = (size_t)S->rows * D.cols;
    if (out) {
        std::vector<double> t(nval);
        if (nval) CK(cudaMemcpy(t.data(), S->tally_d, sizeof(double) * nval, cudaMemcpyDeviceToHost));
        // postProc and / cellVol (montecarlo/problem.cpp:439-444,478-648)
        postProcess(S->desc.problem, S->rows, D.cols, m.energySum, t.data());
        for (long col = 0; col < D.cols; ++col)
            for (int r = 0; r < S->rows; ++r)
                out[(size_t)col * S->rows + r] = S->power * (t[(size_t)col * S->rows + r] / D.cellVol[col]);
    }
    if (S->logging && S->desc.log && S->desc.log_counts) {
        long long ln = std::min<long long>(S->desc.log_phonons, S->nemit);
        std::vector<int> lc(ln);
        CK(cudaMemcpy(S->desc.log, S->log_d, sizeof(double) * 12 * (size_t)ln * S->desc.log_cap, cudaMemcpyDeviceToHost));
        if (ln) CK(cudaMemcpy(lc.data(), S->logcnt_d, sizeof(int) * ln, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < ln; ++i) S->desc.log_counts[i] = lc[i];
        // device slots -> the caller's subdomain indices
        const std::vector<int>& ref = S->dom->refOfSlot;
        for (size_t q = 0; q < (size_t)ln * S->desc.log_cap; ++q) {
            double* r = S->desc.log + 12 * q;
            for (int k : {1, 3}) {
                const double v = r[k];
                if (v >= 0. && v < (double)ref.size()) r[k] = (double)ref[(size_t)v];
            }
        }
    }
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->nemit = S->nemit;
        st->power = S->power;
        st->rows = S->rows;
        st->cols = D.cols;
        st->phonon_steps = (double)c[C_PHONON_STEPS];
        st->events = (long)c[C_EVENTS];
        st->scatters = (long)c[C_SCATTERS];
        st->escapes = (long)c[C_ESCAPES];
        st->horizon_stops = (long)c[C_HORIZON];
        st->maxscat_stops = (long)c[C_MAXSCAT];
        st->maxloop_stops = (long)c[C_MAXLOOP];
        st->absorbed = (long)c[C_ABSORBED];
        st->nonfinite = (long)c[C_BAD];
        st->status = status;
        st->launches = S->launches;
        double cs[4] = {0, 0, 0, 0};
        CK(cudaMemcpy(cs, S->csum_d, sizeof(cs), cudaMemcpyDeviceToHost));
        for (int r = 0; r < 4; ++r) st->checksum[r] = cs[r];
    }
    if (status & S_TIMEOUT) return fail(MC_ERR_TIMEOUT, "a device-side wait exceeded its limit; results discarded");
    if (status & S_REPLAY_EXHAUSTED) return fail(MC_ERR_REPLAY, "replay stream exhausted");
    if (status & S_NONFINITE) return fail(MC_ERR_NONFINITE, "non-finite phonon state");
    return MC_OK;
}

void freeSession(mc_session_s* S) {
    if (!S) return;
    void* ps[] = {S->state, S->tables, S->dom_d, S->em_d, S->cdf_d, S->cnt_d, S->status_d, S->tally_d, S->csum_d,
                  S->rwords_d, S->roff_d, S->rcur_d, S->log_d, S->logcnt_d, S->reg_d};
    for (void* p : ps) {
        if (!p) continue;
        if (S->pooled) cudaFreeAsync(p, S->stream);
        else cudaFree(p);
    }
    if (S->ev0) cudaEventDestroy(S->ev0);
    if (S->ev1) cudaEventDestroy(S->ev1);
    if (S->ownStream && S->stream) cudaStreamDestroy(S->stream);
    delete S;
}

}  // namespace

// ================================================================ batches
struct mc_batch_s {
    int n = 0;
    int prec = 32;
    mc_batch_desc bd{};
    std::vector<mc_material_h> mats;
    std::vector<mc_domain_h> doms;
    std::vector<mc_problem_desc> probs;
    // per instance
    std::vector<void*> tables, sd;
    std::vector<EmitterD*> em;
    std::vector<long long*> cdf;
    std::vector<long> nemit;
    std::vector<double> power;
    std::vector<int> rows, cols;
    std::vector<size_t> fieldOff;   // offset of the instance's field block in `fields`
    // device
    double* fields = nullptr;       // per instance: rows x cols, rows x (cols+1) difference, 4 checksums
    size_t fieldDoubles = 0;
    void* insts = nullptr;
    long long* islot = nullptr;
    void* state = nullptr;
    size_t stateBytes = 0;
    unsigned long long* cnt = nullptr;
    unsigned int* status = nullptr;
    long long cap = 0;
    int block = 256, grid = 0;
    int tm = 2;                     // field mode of the advance launches (batchFieldMode)
    bool gen = false;               // some instance has a subdomain other than the Parallelepiped
    SegD* segs = nullptr;           // work segments of the advance launches
    int* home = nullptr;            // first segment of each block
    unsigned long long* segNext = nullptr;
    int nseg = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
    Params<float> p32{};
    Params<double> p64{};
};

namespace {

// Work segments of a batched advance: instance i's slots split into its
// field copies (groupedId's layout), then each of `grid` blocks given a
// first segment in proportion to the segments' slots.
void planSegments(const std::vector<long long>& slot0, const std::vector<long>& nemit,
                  const std::vector<int>& groups, int grid, std::vector<SegD>& segs, std::vector<int>& home) {
    segs.clear();
    for (size_t i = 0; i < slot0.size(); ++i) {
        const long long n = nemit[i];
        const int G = std::max(1, groups[i]);
        const long long q = n / G, rem = n % G;
        long long off = 0;
        for (int g = 0; g < G; ++g) {
            const long long sz = q + (g < rem ? 1 : 0);
            if (sz > 0) segs.push_back(SegD{slot0[i] + off, slot0[i] + off + sz, (int)i, g});
            off += sz;
        }
    }
    long long total = 0;
    for (const SegD& g : segs) total += g.end - g.beg;
    home.assign((size_t)std::max(grid, 1), 0);
    size_t k = 0;
    long long before = 0;
    for (int b = 0; b < grid && !segs.empty(); ++b) {
        const double pos = ((double)b + 0.5) / (double)grid * (double)total;
        while (k + 1 < segs.size() && (double)(before + (segs[k].end - segs[k].beg)) <= pos) {
            before += segs[k].end - segs[k].beg;
            ++k;
        }
        home[b] = (int)k;
    }
}

// What a batched block stages per instance (InstD::flags) and the launch's
// shared-memory capacities: fixed-point fields up to TAL_BATCH_MAX bytes,
// subdomain images while the block stays within BATCH_SMEM_F32 (twice that
// in FP64). `inst` must hold nw, np, nsd, rows and cols.
// The field mode every instance of a batched launch shares (so the launch
// runs the kernel without the others' code), or TM_AUTO.
template <typename R>
int batchFieldMode(const std::vector<InstD<R>>& inst) {
    bool allShared = true, allGlobal = true, allNone = true;
    for (const auto& I : inst) {
        const bool none = (I.flags & IF_NO_FIELD) != 0 || I.tally == nullptr;
        const bool sh = !none && (I.flags & IF_TAL_SHARED) != 0;
        allNone = allNone && none;
        allShared = allShared && sh;
        allGlobal = allGlobal && !none && !sh;
    }
    return allNone ? TM_NONE : (allShared ? TM_SHARED : (allGlobal ? TM_GLOBAL : TM_AUTO));
}

template <typename R>
int batchCaps(std::vector<InstD<R>>& inst, Params<R>& P) {
    int bNt = 0, bNw = 0, bTal = 0;
    for (auto& I : inst) {
        bNt = std::max(bNt, I.nw * I.np);
        bNw = std::max(bNw, I.nw);
        const size_t talE = talEntries(I.rows, (int)I.cols);
        I.flags = 0;
        if (talE * sizeof(long long) <= TAL_BATCH_MAX) {
            I.flags |= IF_TAL_SHARED;
            bTal = std::max(bTal, (int)talE);
        }
    }
    BatchSmem L;
    L.init<R>(bNt, bNw, 0, bTal);
    const size_t limit = sizeof(R) == 4 ? BATCH_SMEM_F32 : 2 * BATCH_SMEM_F32;
    const size_t budget = L.total < limit ? limit - L.total : 0;
    int bSd = 0;
    for (auto& I : inst) {
        const size_t sdB = sizeof(SdomD<R>) * (size_t)I.nsd;
        if (sdB <= budget && sdB <= SD_SHARED_MAX) {
            I.flags |= IF_SD_SHARED;
            bSd = std::max(bSd, (int)sdB);
        }
    }
    P.bNt = bNt; P.bNw = bNw; P.bTal = bTal; P.bSdBytes = bSd;
    setBatchLayout(P);
    if (batchSmemBytes<R>(P) > 227 * 1024) return fail(MC_ERR_UNSUPPORTED, "batched shared-memory tables exceed 227 KB");
    return MC_OK;
}

void freeBatch(mc_batch_s* B) {
    if (!B) return;
    for (void* p : B->tables) if (p) cudaFree(p);
    for (void* p : B->sd) if (p) cudaFree(p);
    for (auto* p : B->em) if (p) cudaFree(p);
    for (auto* p : B->cdf) if (p) cudaFree(p);
    void* ps[] = {B->fields, B->insts, B->islot, B->state, B->cnt, B->status, B->segs, B->home, B->segNext};
    for (void* p : ps) if (p) cudaFree(p);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->ownStream && B->stream) cudaStreamDestroy(B->stream);
    delete B;
}

template <typename R>
Params<R>& batchParams(mc_batch_s* B);
template <> Params<float>& batchParams<float>(mc_batch_s* B) { return B->p32; }
template <> Params<double>& batchParams<double>(mc_batch_s* B) { return B->p64; }

template <typename R>
int setupBatch(mc_batch_s* B) {
    const int n = B->n;
    B->tables.assign(n, nullptr); B->sd.assign(n, nullptr); B->em.assign(n, nullptr); B->cdf.assign(n, nullptr);
    B->nemit.assign(n, 0); B->power.assign(n, 0.); B->rows.assign(n, 1); B->cols.assign(n, 0);
    B->fieldOff.assign(n, 0);
    std::vector<InstD<R>> inst(n);
    std::vector<long long> islot(n + 1, 0);
    const int K = B->bd.steps_per_launch > 0 ? B->bd.steps_per_launch : (int)B->bd.nsteps;
    const double window = (double)std::min<long>(K, B->bd.nsteps) * B->bd.dt;
    // fields: one allocation
    size_t off = 0;
    for (int i = 0; i < n; ++i) {
        const mc_problem_desc& p = B->probs[i];
        B->rows[i] = (int)problemRows(p.problem, p.cum_size);
        B->cols[i] = (int)B->doms[i]->cols;
        B->fieldOff[i] = off;
        off += (size_t)B->rows[i] * B->cols[i] + (size_t)B->rows[i] * (B->cols[i] + 1) + 4;
    }
    B->fieldDoubles = off;
    CK(cudaMalloc(&B->fields, sizeof(double) * std::max<size_t>(off, 1)));
    for (int i = 0; i < n; ++i) {
        const mc_material_s& m = *B->mats[i];
        const mc_domain_s& D = *B->doms[i];
        const mc_problem_desc& pd = B->probs[i];
        Params<R> P{};
        double vmax = 0.;
        int rc = uploadMaterial<R>(m, &B->tables[i], P, vmax);
        if (rc) return rc;
        rc = uploadDomain<R>(D, m.fluxSum, pd.nemit, &B->sd[i], &B->em[i], &B->cdf[i], P, B->nemit[i], B->power[i]);
        if (rc) return rc;
        islot[i + 1] = islot[i] + B->nemit[i];
        InstD<R>& I = inst[i];
        std::memset(&I, 0, sizeof(I));
        I.vel = P.vel; I.vt = P.vt; I.wthr = P.wthr; I.wguide = P.wguide; I.pthr = P.pthr;
        I.fwthr = P.fwthr; I.fpthr = P.fpthr;
        I.sd = P.sd; I.em = P.em; I.emitCdf = P.emitCdf;
        I.nw = P.nw; I.np = P.np; I.nem = P.nem; I.nsd = P.nsd;
        I.problem = pd.problem; I.rows = B->rows[i]; I.cols = B->cols[i]; I.inst = i;
        I.cumStep = cumStepOf(pd.problem, pd.maxscat, pd.cum_size);
        I.maxscat = pd.maxscat;
        I.maxloop = pd.maxloop != 0 ? pd.maxloop : 100 * pd.maxscat;
        I.slot0 = islot[i]; I.nemit = B->nemit[i];
        I.key0 = (uint32_t)pd.seed; I.key1 = (uint32_t)(pd.seed >> 32);
        double* f = B->fields + B->fieldOff[i];
        I.tally = f;
        bool oneD = false;
        for (const auto& sd : D.sd) oneD = oneD || (sd.accum >= 0 && sd.accum <= 2);
        I.gdif = oneD ? f + (size_t)I.rows * I.cols : nullptr;
        I.csum = f + (size_t)I.rows * I.cols + (size_t)I.rows * (I.cols + 1);
        I.groups = 1;
        I.gstride = 0;
        // a block's shared field takes at most the instance's phonons
        for (int r = 0; r < 4; ++r) {
            const double q = tallyQuantum(sizeof(R) == 4, window * (timeClass(pd.problem, r) ? 1.0 : vmax), (double)B->nemit[i]);
            I.tq[r] = q;
            I.tqinv[r] = (R)(1.0 / q);
        }
        if (pd.maxscat <= 0 || pd.maxloop < 0 || pd.nemit <= 0) return fail(MC_ERR_ARG, "Invalid problem arguments");
        if (int rcp = checkProblem(pd)) return rcp;
    }
    B->cap = islot[n];
    Params<R>& P = batchParams<R>(B);
    P = Params<R>{};
    {
        int rc = batchCaps<R>(inst, P);
        if (rc) return rc;
        for (auto& I : inst)
            if (I.flags & IF_TAL_SHARED) I.gdif = nullptr;
    }
    CK(cudaMalloc(&B->insts, sizeof(InstD<R>) * n));
    CK(cudaMemcpy(B->insts, inst.data(), sizeof(InstD<R>) * n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&B->islot, sizeof(long long) * (n + 1)));
    CK(cudaMemcpy(B->islot, islot.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice));
    // state: one half, updated in place
    using V4 = typename Vec4<R>::T;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t cap = (size_t)B->cap;
    B->stateBytes = (2 * sizeof(V4) + sizeof(uint4)) * cap;
    CK(cudaMalloc(&B->state, 2 * al(sizeof(V4) * cap) + al(sizeof(uint4) * cap)));
    char* sb = (char*)B->state;
    P.P0in = P.P0out = (V4*)sb; sb += al(sizeof(V4) * cap);
    P.P1in = P.P1out = (V4*)sb; sb += al(sizeof(V4) * cap);
    P.P2in = P.P2out = (uint4*)sb;
    CK(cudaMalloc(&B->cnt, sizeof(unsigned long long) * (C_NCOUNTERS + 4)));
    CK(cudaMalloc(&B->status, sizeof(unsigned int)));
    P.counters = B->cnt;
    P.status = B->status;
    P.live_in = B->cnt + C_NCOUNTERS;
    P.live_out = B->cnt + C_NCOUNTERS + 1;
    P.cap = (unsigned long long)cap;
    P.dt = (R)B->bd.dt;
    P.nsteps = (int)B->bd.nsteps;
    P.ksteps = K;
    P.insts = (const InstD<R>*)B->insts;
    P.islot = B->islot;
    P.ninst = n;
    P.maxGroups = 1;
    P.maxRows = 1;
    for (int i = 0; i < n; ++i) P.maxRows = std::max(P.maxRows, B->rows[i]);
    B->block = B->bd.block_size > 0 ? B->bd.block_size : 256;
    if (B->block % 32 || B->block > 256) return fail(MC_ERR_ARG, "block_size must be a multiple of 32, <= 256");
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    B->tm = batchFieldMode<R>(inst);
    B->gen = false;
    for (int i = 0; i < n; ++i) B->gen = B->gen || B->doms[i]->needGen;
    const int occ = advanceBatchOccupancy<R>(B->tm, B->gen, batchSmemBytes<R>(P), B->block);
    if (occ <= 0) return fail(MC_ERR_UNSUPPORTED, "batched kernel cannot launch with this configuration");
    B->grid = B->bd.grid_blocks > 0 ? B->bd.grid_blocks : occ * nsm;
    std::vector<SegD> segs;
    std::vector<int> home;
    std::vector<long long> slot0(islot.begin(), islot.end() - 1);
    planSegments(slot0, B->nemit, std::vector<int>(n, 1), B->grid, segs, home);
    B->nseg = (int)segs.size();
    CK(cudaMalloc(&B->segs, sizeof(SegD) * std::max<size_t>(segs.size(), 1)));
    CK(cudaMalloc(&B->home, sizeof(int) * home.size()));
    CK(cudaMalloc(&B->segNext, sizeof(unsigned long long) * std::max<size_t>(segs.size(), 1)));
    if (!segs.empty()) CK(cudaMemcpy(B->segs, segs.data(), sizeof(SegD) * segs.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B->home, home.data(), sizeof(int) * home.size(), cudaMemcpyHostToDevice));
    P.segs = B->segs;
    P.home = B->home;
    P.segNext = B->segNext;
    P.nseg = B->nseg;
    return MC_OK;
}

// The launch sequence of one batched run (captured into a graph or issued
// directly).
template <typename R>
int enqueueBatch(mc_batch_s* B) {
    Params<R> P = batchParams<R>(B);
    CK(cudaMemsetAsync(B->fields, 0, sizeof(double) * B->fieldDoubles, B->stream));
    CK(cudaMemsetAsync(B->cnt, 0, sizeof(unsigned long long) * (C_NCOUNTERS + 4), B->stream));
    CK(cudaMemsetAsync(B->status, 0, sizeof(unsigned int), B->stream));
    CK(launchEmitBatch<R>(P, B->stream));
    int launches = 1;
    for (int step = 0; step < (int)B->bd.nsteps; step += P.ksteps) {
        P.step0 = step;
        setWindow(P);
        CK(cudaMemsetAsync(B->cnt + C_NCOUNTERS + 1, 0, sizeof(unsigned long long), B->stream));
        CK(cudaMemsetAsync(B->segNext, 0, sizeof(unsigned long long) * std::max(B->nseg, 1), B->stream));
        CK(launchAdvanceBatch<R>(P, B->tm, B->gen, B->grid, B->block, B->stream));
        ++launches;
    }
    CK(launchDifPrefix<R>(P, B->stream));
    B->launches = launches + 1;
    return MC_OK;
}

template <typename R>
int runBatch(mc_batch_s* B) {
    if (!B->bd.use_graph) return enqueueBatch<R>(B);
    if (!B->exec) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueueBatch<R>(B);
        cudaError_t e = cudaStreamEndCapture(B->stream, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return cudaFail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&B->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cudaFail(e, "cudaGraphInstantiate");
    }
    CK(cudaGraphLaunch(B->exec, B->stream));
    return MC_OK;
}

int batchCounters(mc_batch_s* B, mc_stats* st) {
    CK(cudaStreamSynchronize(B->stream));
    std::vector<unsigned long long> c(C_NCOUNTERS + 4);
    unsigned int status = 0;
    CK(cudaMemcpy(c.data(), B->cnt, sizeof(unsigned long long) * c.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&status, B->status, sizeof(status), cudaMemcpyDeviceToHost));
    std::memset(st, 0, sizeof(*st));
    st->nemit = (long)B->cap;
    st->phonon_steps = (double)c[C_PHONON_STEPS];
    st->events = (long)c[C_EVENTS];
    st->scatters = (long)c[C_SCATTERS];
    st->escapes = (long)c[C_ESCAPES];
    st->horizon_stops = (long)c[C_HORIZON];
    st->maxscat_stops = (long)c[C_MAXSCAT];
    st->maxloop_stops = (long)c[C_MAXLOOP];
    st->absorbed = (long)c[C_ABSORBED];
    st->nonfinite = (long)c[C_BAD];
    st->status = status;
    st->launches = B->launches;
    if (status & S_NONFINITE) return fail(MC_ERR_NONFINITE, "non-finite phonon state");
    return MC_OK;
}

}  // namespace

// ================================================================ serving
namespace {

using Clock = std::chrono::steady_clock;

// Phonons per emitter for a requested count (montecarlo/problem.cpp:315-342,
// as in uploadDomain): cumulative counts into cdf, returns the total.
long long allocEmitters(const std::vector<double>& w, long nemitReq, std::vector<long long>& cdf) {
    double wsum = 0.;
    for (double x : w) wsum += x;
    cdf.assign(w.size(), 0);
    long long tot = 0;
    for (size_t i = 0; i < w.size(); ++i) {
        const double rounded = std::ceil(w[i] / wsum * nemitReq - 0.5);
        tot += std::max(1LL, (long long)rounded);
        cdf[i] = tot;
    }
    return tot;
}

// State slots are handed out in multiples of this many (aligned warps).
constexpr long long SLOT_ALIGN = 64;
long long slotsFor(long long phonons) { return (phonons + SLOT_ALIGN - 1) / SLOT_ALIGN * SLOT_ALIGN; }

// Free ranges of the server's state buffer: first fit, neighbours merged.
struct SlotPool {
    std::map<long long, long long> freeR;  // start -> length
    void init(long long cap) {
        freeR.clear();
        if (cap > 0) freeR[0] = cap;
    }
    long long take(long long n) {
        for (auto it = freeR.begin(); it != freeR.end(); ++it) {
            if (it->second < n) continue;
            const long long s = it->first, len = it->second;
            freeR.erase(it);
            if (len > n) freeR[s + n] = len - n;
            return s;
        }
        return -1;
    }
    void give(long long s, long long n) {
        auto it = freeR.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != freeR.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            freeR.erase(nx);
        }
        if (it != freeR.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                freeR.erase(it);
            }
        }
    }
};

// One submitted solve.
struct SrvJob {
    long ticket = 0;
    mc_request req{};
    double tSubmit = 0., tAdmit = -1., tDone = -1.;
    // resident device data
    void* tables = nullptr;
    void* sd = nullptr;
    EmitterD* em = nullptr;
    long long* cdf = nullptr;
    double* fields = nullptr;  // groups x [tally rows*cols | difference rows*(cols+1)], then groups x 4 checksums
    double* acc = nullptr;     // running sum of the rounds' fields, rows*cols (field requests)
    long nemit = 0;            // phonons of the current round
    long nextReq = 0;          // requested phonons of the next round
    double wflux = 0.;         // power x phonons of a round: sum of emitter weights x fluxSum / 4
    double vmax = 0.;
    int rows = 1, cols = 0, fluxRow0 = 0;
    bool oneD = false;
    double grad = 0., volume = 0.;
    std::vector<double> emW;   // emitter weights
    unsigned char image[512];  // host InstD<R> without the per-tick fields
    // the current round's state slots [slot0, slot0 + slots), -1 between
    // rounds, and the windows of it already run
    long long slot0 = -1, slots = 0;
    int window = 0;
    int maxRounds = 0;
    bool cancel = false;
    // pooled batch-mean statistics over rounds of unequal size: round r
    // gives `groups` estimates from N_r / groups phonons each
    long rounds = 0;
    double sumN = 0., sumNK = 0., ss = 0., steps = 0.;
    long dof = 0;
    int status = MC_OK;
    bool done = false;
    std::vector<double> field;  // mean field at completion
    double kappa() const { return sumN > 0. ? sumNK / sumN : 0.; }
    double se() const { return dof > 0 && sumN > 0. ? std::sqrt(ss / (double)dof / sumN) : 1e300; }
};

struct ServerBase {
    virtual ~ServerBase() = default;
    virtual void loop() = 0;
    mc_server_desc d{};
    int dev = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv, cvDone;
    std::deque<SrvJob*> pending;
    std::vector<SrvJob*> active;  // in ticket order
    std::map<long, SrvJob*> jobs;
    long nextTicket = 1;
    long long capacity = 0;       // phonon slots of the state buffer
    SlotPool pool;
    bool stop = false;
    mc_server_counters st{};
    std::thread th;
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

void freeJobDevice(SrvJob* j) {
    void* ps[] = {j->tables, j->sd, j->em, j->cdf, j->fields, j->acc};
    for (void* p : ps) if (p) cudaFree(p);
    j->tables = j->sd = nullptr; j->em = nullptr; j->cdf = nullptr; j->fields = nullptr; j->acc = nullptr;
}

template <typename R>
struct ServerT : ServerBase {
    void* state = nullptr;
    unsigned long long* cnt = nullptr;
    unsigned int* status = nullptr;
    InstD<R>* insts_d = nullptr;   // every solve of a tick
    InstD<R>* starts_d = nullptr;  // the solves whose round starts in the tick
    long long* islot_d = nullptr;  // emission ranges of those
    double** accs_d = nullptr;
    double* gsum_d = nullptr;
    SegD* segs_d = nullptr;
    int* home_d = nullptr;
    unsigned long long* segNext_d = nullptr;
    cudaStream_t stream = nullptr;
    int block = 256, nsm = 0;
    int K = 0, nwin = 1;            // dt-steps per window, windows per round
    long maxRound = 0;              // largest round a solve grows to (a server constant)
    Params<R> base{};

    int init() {
        CK(cudaGetDevice(&dev));
        if (d.steps_per_window < 0 || d.steps_per_window > d.nsteps || (d.steps_per_window > 0 && d.nsteps % d.steps_per_window))
            return fail(MC_ERR_ARG, "steps_per_window must divide nsteps");
        K = d.steps_per_window;
        if (K == 0) {
            // two windows per round: measured on the served stream against an
            // eighth and a quarter of the horizon, it gave both the most
            // solves/s at saturation and the lowest latencies below it (each
            // tick's emission, flush and reduction cost less per phonon-step)
            K = (int)std::max(1L, d.nsteps / 2);
            while (d.nsteps % K) --K;
        }
        nwin = (int)(d.nsteps / K);
        using V4 = typename Vec4<R>::T;
        const size_t per = 2 * sizeof(V4) + sizeof(uint4);
        capacity = (long long)(d.hbm_budget / per) / SLOT_ALIGN * SLOT_ALIGN;
        if (capacity < 1024) return fail(MC_ERR_ARG, "hbm_budget too small");
        maxRound = std::max(1LL, capacity / 4 - SLOT_ALIGN);
        pool.init(capacity);
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        const size_t cap = (size_t)capacity;
        CK(cudaMalloc(&state, 2 * al(sizeof(V4) * cap) + al(sizeof(uint4) * cap)));
        char* sb = (char*)state;
        base.P0in = base.P0out = (V4*)sb; sb += al(sizeof(V4) * cap);
        base.P1in = base.P1out = (V4*)sb; sb += al(sizeof(V4) * cap);
        base.P2in = base.P2out = (uint4*)sb;
        CK(cudaMalloc(&cnt, sizeof(unsigned long long) * (C_NCOUNTERS + 4)));
        CK(cudaMalloc(&status, sizeof(unsigned int)));
        CK(cudaMalloc(&insts_d, sizeof(InstD<R>) * d.max_active));
        CK(cudaMalloc(&starts_d, sizeof(InstD<R>) * d.max_active));
        CK(cudaMalloc(&islot_d, sizeof(long long) * (d.max_active + 1)));
        CK(cudaMalloc(&accs_d, sizeof(double*) * d.max_active));
        CK(cudaMalloc(&gsum_d, sizeof(double) * d.max_active * MAX_GROUPS * 4));
        CK(cudaMalloc(&segs_d, sizeof(SegD) * d.max_active * MAX_GROUPS));
        CK(cudaMalloc(&segNext_d, sizeof(unsigned long long) * d.max_active * MAX_GROUPS));
        base.counters = cnt;
        base.status = status;
        base.live_in = cnt + C_NCOUNTERS;
        base.live_out = cnt + C_NCOUNTERS + 1;
        base.dt = (R)d.dt;
        base.nsteps = (int)d.nsteps;
        base.ksteps = K;
        base.step0 = 0;
        base.maxGroups = d.groups;
        base.maxRows = 4;
        block = d.block_size > 0 ? d.block_size : 256;
        if (block % 32 || block > 256) return fail(MC_ERR_ARG, "block_size must be a multiple of 32, <= 256");
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        // at most 2048 / 32 blocks of a warp or more per SM
        CK(cudaMalloc(&home_d, sizeof(int) * (size_t)nsm * 64));
        return MC_OK;
    }

    ~ServerT() override {
        void* ps[] = {state, cnt, status, insts_d, starts_d, islot_d, accs_d, gsum_d, segs_d, home_d, segNext_d};
        for (void* p : ps) if (p) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    // Phonons of a request's first round (the emitter rounding of its
    // requested count), known before anything is uploaded.
    long long firstRound(const SrvJob* j) const {
        std::vector<long long> cdf;
        return allocEmitters(j->req.dom->emWeight, j->req.nemit, cdf);
    }

    // Size the job's next round at `want` requested phonons: emitter counts,
    // the instance image's phonon count and fixed-point quanta.
    int setRound(SrvJob* j, long want) {
        std::vector<long long> cdf;
        const long long tot = allocEmitters(j->emW, want, cdf);
        CK(cudaMemcpyAsync(j->cdf, cdf.data(), sizeof(long long) * cdf.size(), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));  // cdf lives on this stack
        j->nemit = (long)tot;
        InstD<R> I;
        std::memcpy(&I, j->image, sizeof(I));
        I.nemit = j->nemit;
        // a flight stays inside one window: the window bounds its amount
        const double window = (double)K * d.dt;
        // a block's shared field takes at most one field copy's phonons
        const double perCopy = (double)((j->nemit + d.groups - 1) / d.groups);
        for (int r = 0; r < 4; ++r) {
            const bool timeRow = j->req.problem == MC_MULTI && r == 0;
            const double q = tallyQuantum(sizeof(R) == 4, window * (timeRow ? 1.0 : j->vmax), perCopy);
            I.tq[r] = q;
            I.tqinv[r] = (R)(1.0 / q);
        }
        std::memcpy(j->image, &I, sizeof(I));
        return MC_OK;
    }

    // upload a job's tables and domain, allocate its fields
    int admit(SrvJob* j) {
        const mc_material_s& m = *j->req.mat;
        const mc_domain_s& D = *j->req.dom;
        Params<R> P{};
        int rc = uploadMaterial<R>(m, &j->tables, P, j->vmax);
        if (rc) return rc;
        double power = 0.;
        rc = uploadDomain<R>(D, m.fluxSum, j->req.nemit, &j->sd, &j->em, &j->cdf, P, j->nemit, power);
        if (rc) return rc;
        j->emW = D.emWeight;
        j->wflux = power * (double)j->nemit;
        j->rows = j->req.problem == MC_FLUX ? 3 : 4;
        j->fluxRow0 = j->req.problem == MC_FLUX ? 0 : 1;
        j->cols = (int)D.cols;
        for (const auto& s : D.sd) j->oneD = j->oneD || (s.accum >= 0 && s.accum <= 2);
        const size_t gstride = (size_t)j->rows * j->cols + (size_t)j->rows * (j->cols + 1);
        const bool wantField = j->req.field != 0;
        CK(cudaMalloc(&j->fields, sizeof(double) * (wantField ? gstride * d.groups : 0) + sizeof(double) * 4 * d.groups));
        if (wantField) {
            CK(cudaMalloc(&j->acc, sizeof(double) * (size_t)j->rows * j->cols));
            CK(cudaMemset(j->acc, 0, sizeof(double) * (size_t)j->rows * j->cols));
        }
        double vol = 0.;
        for (double v : D.cellVol) vol += v;
        j->volume = j->req.volume > 0. ? j->req.volume : vol;
        j->grad = j->req.gradient != 0. ? j->req.gradient : D.desc[0].gradT[j->req.axis];
        if (!(j->grad != 0.) || !std::isfinite(j->grad)) return fail(MC_ERR_ARG, "no temperature gradient along the kappa axis");
        InstD<R> I;
        std::memset(&I, 0, sizeof(I));
        I.vel = P.vel; I.vt = P.vt; I.wthr = P.wthr; I.wguide = P.wguide; I.pthr = P.pthr;
        I.fwthr = P.fwthr; I.fpthr = P.fpthr;
        I.sd = P.sd; I.em = P.em; I.emitCdf = P.emitCdf;
        I.nw = P.nw; I.np = P.np; I.nem = P.nem; I.nsd = P.nsd;
        I.problem = j->req.problem; I.rows = j->rows; I.cols = wantField ? j->cols : 0;
        I.maxscat = j->req.maxscat;
        I.maxloop = j->req.maxloop != 0 ? j->req.maxloop : 100 * j->req.maxscat;
        I.tally = wantField ? j->fields : nullptr;
        I.gdif = wantField && j->oneD ? j->fields + (size_t)j->rows * j->cols : nullptr;
        I.csum = j->fields + (wantField ? gstride * d.groups : 0);
        I.groups = d.groups;
        I.gstride = wantField ? (long long)gstride : 0;
        static_assert(sizeof(InstD<R>) <= sizeof(j->image), "instance image");
        std::memcpy(j->image, &I, sizeof(I));
        j->nextReq = j->req.nemit;
        j->window = 0;
        return setRound(j, j->req.nemit);
    }

    // One window of every running solve: emission of the rounds that start
    // now, one batched advance launch over all of them, and for the rounds
    // that end with it the field finish and their batch-mean statistics.
    int tick(const std::vector<SrvJob*>& run) {
        const int n = (int)run.size();
        std::vector<InstD<R>> inst(n);
        std::vector<double*> accs(n);
        std::vector<int> starts;
        for (int i = 0; i < n; ++i) {
            SrvJob* j = run[i];
            std::memcpy(&inst[i], j->image, sizeof(InstD<R>));
            inst[i].inst = i;
            inst[i].slot0 = j->slot0;
            const uint64_t seed = j->req.seed + (uint64_t)j->rounds;
            inst[i].key0 = (uint32_t)seed;
            inst[i].key1 = (uint32_t)(seed >> 32);
            accs[i] = j->acc;
            if (j->window == 0) {
                starts.push_back(i);
                const size_t fieldD = (size_t)inst[i].gstride * d.groups + 4 * (size_t)d.groups;
                CK(cudaMemsetAsync(j->fields, 0, sizeof(double) * fieldD, stream));
            }
        }
        Params<R> P = base;
        {
            int rc = batchCaps<R>(inst, P);
            if (rc) return rc;
            for (int i = 0; i < n; ++i) {
                InstD<R>& I = inst[i];
                if (I.flags & IF_TAL_SHARED) I.gdif = nullptr;
                if (I.tally == nullptr) I.flags |= IF_NO_FIELD;
                if (run[i]->window + 1 == nwin) I.flags |= IF_LAST;
            }
        }
        const int tm = batchFieldMode<R>(inst);
        bool gen = false;
        for (SrvJob* j : run) gen = gen || j->req.dom->needGen;
        const int occ = advanceBatchOccupancy<R>(tm, gen, batchSmemBytes<R>(P), block);
        if (occ <= 0) return fail(MC_ERR_UNSUPPORTED, "batched kernel cannot launch with this configuration");
        const int grid = std::min(occ, 64) * nsm;
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (C_NCOUNTERS + 4), stream));
        CK(cudaMemsetAsync(status, 0, sizeof(unsigned int), stream));
        CK(cudaMemcpyAsync(insts_d, inst.data(), sizeof(InstD<R>) * n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(accs_d, accs.data(), sizeof(double*) * n, cudaMemcpyHostToDevice, stream));
        std::vector<InstD<R>> sinst;
        std::vector<long long> sslot(1, 0);
        for (int i : starts) {
            sinst.push_back(inst[i]);
            sslot.push_back(sslot.back() + run[i]->nemit);
        }
        if (!starts.empty()) {
            // emission of the starting rounds into their own slots
            CK(cudaMemcpyAsync(starts_d, sinst.data(), sizeof(InstD<R>) * sinst.size(), cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(islot_d, sslot.data(), sizeof(long long) * sslot.size(), cudaMemcpyHostToDevice, stream));
            Params<R> E = P;
            E.insts = starts_d;
            E.islot = islot_d;
            E.ninst = (int)starts.size();
            E.cap = (unsigned long long)sslot.back();
            CK(launchEmitBatch<R>(E, stream));
        }
        std::vector<SegD> segs;
        std::vector<int> home;
        std::vector<long long> slot0(n);
        std::vector<long> nem(n);
        for (int i = 0; i < n; ++i) { slot0[i] = run[i]->slot0; nem[i] = run[i]->nemit; }
        planSegments(slot0, nem, std::vector<int>(n, d.groups), grid, segs, home);
        if (!segs.empty())
            CK(cudaMemcpyAsync(segs_d, segs.data(), sizeof(SegD) * segs.size(), cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(home_d, home.data(), sizeof(int) * home.size(), cudaMemcpyHostToDevice, stream));
        CK(cudaMemsetAsync(segNext_d, 0, sizeof(unsigned long long) * std::max<size_t>(segs.size(), 1), stream));
        P.segs = segs_d;
        P.home = home_d;
        P.segNext = segNext_d;
        P.nseg = (int)segs.size();
        P.insts = insts_d;
        P.ninst = n;
        P.lastOnly = 1;
        setWindow(P);
        CK(launchAdvanceBatch<R>(P, tm, gen, grid, block, stream));
        CK(launchDifPrefix<R>(P, stream));
        CK(launchRoundReduce<R>(P, accs_d, gsum_d, stream));
        std::vector<double> gsum((size_t)n * MAX_GROUPS * 4);
        std::vector<unsigned long long> c(C_NCOUNTERS + 4);
        unsigned int stat = 0;
        CK(cudaMemcpyAsync(gsum.data(), gsum_d, sizeof(double) * gsum.size(), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(c.data(), cnt, sizeof(unsigned long long) * c.size(), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(&stat, status, sizeof(stat), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (stat & S_NONFINITE) return fail(MC_ERR_NONFINITE, "non-finite phonon state");
        st.phonon_steps += (double)c[C_PHONON_STEPS];
        const int G = d.groups;
        for (int i = 0; i < n; ++i) {
            SrvJob* j = run[i];
            if (++j->window < nwin) continue;
            j->rounds++;
            // group g holds N / G phonons: kappa_g = -G power q_g / (V gradT)
            const double N = (double)j->nemit;
            double k[MAX_GROUPS], kbar = 0.;
            for (int g = 0; g < G; ++g) {
                const double q = (double)G * (j->wflux / N) * gsum[((size_t)i * MAX_GROUPS + g) * 4 + j->fluxRow0 + j->req.axis] /
                                 j->volume;
                k[g] = -q / j->grad;
                kbar += k[g] / (double)G;
            }
            for (int g = 0; g < G; ++g) j->ss += N / (double)G * (k[g] - kbar) * (k[g] - kbar);
            j->dof += G - 1;
            j->sumN += N;
            j->sumNK += N * kbar;
            j->steps += N * (double)d.nsteps;
        }
        return MC_OK;
    }

    // Result of a finished solve; frees its device data (outside the lock).
    void complete(SrvJob* j, int status) {
        j->status = status;
        // mean field over the rounds' phonons: (power x N) / sum N x sum of
        // the rounds' tallies, post-processed (montecarlo/problem.cpp:439-444)
        const mc_material_s& m = *j->req.mat;
        const mc_domain_s& D = *j->req.dom;
        if (j->acc && j->rounds > 0) {
            std::vector<double> a((size_t)j->rows * j->cols, 0.);
            cudaMemcpy(a.data(), j->acc, sizeof(double) * a.size(), cudaMemcpyDeviceToHost);
            j->field.assign(a.size(), 0.);
            for (int c = 0; c < j->cols; ++c)
                for (int r = 0; r < j->rows; ++r) {
                    double v = a[(size_t)c * j->rows + r];
                    if (j->req.problem == MC_MULTI && r == 0) v /= m.energySum;
                    j->field[(size_t)c * j->rows + r] = j->wflux / j->sumN * (v / D.cellVol[c]);
                }
        }
        freeJobDevice(j);
    }

    // Phonons of the job's next round: the estimated remainder to reach the
    // target error (10% margin), at least the requested round, and at most
    // the larger of the requested round and a quarter of the budget.
    long nextRound(const SrvJob* j) const {
        const double target = d.target_rel_se * std::fabs(j->kappa());
        const double se = j->se();
        double need = (double)j->req.nemit;
        if (target > 0. && se < 1e299) need = j->sumN * ((se / target) * (se / target) * 1.1 - 1.0);
        need = std::max(need, (double)j->req.nemit);
        return (long)std::min(need, (double)std::max(maxRound, j->req.nemit));
    }

    // (under the lock) state slots for a round of `phonons`
    bool takeSlots(SrvJob* j, long long phonons) {
        const long long n = slotsFor(phonons);
        const long long s = pool.take(n);
        if (s < 0) return false;
        j->slot0 = s;
        j->slots = n;
        return true;
    }
    void releaseSlots(SrvJob* j) {
        if (j->slot0 >= 0) pool.give(j->slot0, j->slots);
        j->slot0 = -1;
        j->slots = 0;
    }

    // (under the lock) publish a finished solve
    void publish(SrvJob* j) {
        j->tDone = now();
        j->done = true;
        st.completed++;
    }

    void loop() override {
        cudaSetDevice(dev);
        for (;;) {
            std::vector<SrvJob*> toAdmit, dropped, run;
            std::vector<int> droppedRc;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (stop) break;
                // cancellations of admitted solves take effect between windows
                std::vector<SrvJob*> keep;
                for (SrvJob* j : active) {
                    if (j->cancel) {
                        releaseSlots(j);
                        dropped.push_back(j);
                        droppedRc.push_back(MC_ERR_CANCELLED);
                    } else {
                        keep.push_back(j);
                    }
                }
                active.swap(keep);
                // slots for the next round of the solves between rounds,
                // oldest first; then new requests while nobody older waits
                bool blocked = false;
                for (SrvJob* j : active) {
                    if (j->slot0 >= 0) continue;
                    if (!takeSlots(j, j->nemit)) { blocked = true; break; }
                }
                while (!blocked && !pending.empty() && (int)(active.size() + toAdmit.size()) < d.max_active) {
                    SrvJob* j = pending.front();
                    const long long n = firstRound(j);
                    if (slotsFor(n) > capacity) {
                        // can never fit: refused alone
                        pending.pop_front();
                        dropped.push_back(j);
                        droppedRc.push_back(fail(MC_ERR_BUSY, "request larger than the HBM budget"));
                        continue;
                    }
                    if (!takeSlots(j, n)) break;
                    pending.pop_front();
                    toAdmit.push_back(j);
                }
                if (active.empty() && toAdmit.empty() && dropped.empty()) {
                    cv.wait_for(lk, std::chrono::milliseconds(5));
                    continue;
                }
            }
            for (size_t k = 0; k < dropped.size(); ++k) complete(dropped[k], droppedRc[k]);
            std::vector<int> admitRc(toAdmit.size());
            for (size_t k = 0; k < toAdmit.size(); ++k) {
                SrvJob* j = toAdmit[k];
                j->maxRounds = j->req.max_rounds > 0 ? j->req.max_rounds : d.max_rounds;
                admitRc[k] = admit(j);
                if (admitRc[k]) complete(j, admitRc[k]);
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                for (SrvJob* j : dropped) publish(j);
                for (size_t k = 0; k < toAdmit.size(); ++k) {
                    SrvJob* j = toAdmit[k];
                    if (admitRc[k]) {
                        releaseSlots(j);
                        publish(j);
                        continue;
                    }
                    j->tAdmit = now();
                    active.push_back(j);
                    st.admitted++;
                }
                for (SrvJob* j : active)
                    if (j->slot0 >= 0) run.push_back(j);
                if (!dropped.empty() || !toAdmit.empty()) cvDone.notify_all();
            }
            if (run.empty()) continue;
            const double tb = now();
            const int rc = tick(run);
            // each solve whose round ended: converged, out of rounds, or the
            // next round sized (outside the lock: setRound copies)
            std::vector<int> fate(run.size(), 0);  // 0 going on, 1 converged, 2 gave up, 3 error
            for (size_t i = 0; i < run.size(); ++i) {
                SrvJob* j = run[i];
                if (rc) { fate[i] = 3; continue; }
                if (j->window < nwin) continue;
                j->window = 0;
                const bool conv = j->rounds >= d.min_rounds && j->se() <= d.target_rel_se * std::fabs(j->kappa());
                if (conv) fate[i] = 1;
                else if (j->rounds >= j->maxRounds) fate[i] = 2;
                else {
                    fate[i] = 4;  // between rounds
                    const long want = nextRound(j);
                    if (want != j->nextReq) {
                        j->nextReq = want;
                        if (setRound(j, want)) fate[i] = 3;
                    }
                }
            }
            for (size_t i = 0; i < run.size(); ++i)
                if (fate[i] >= 1 && fate[i] <= 3)
                    complete(run[i], fate[i] == 1 ? MC_OK : (fate[i] == 2 ? MC_ERR_BUSY : (rc ? rc : MC_ERR_CUDA)));
            std::lock_guard<std::mutex> lk(mu);
            st.ticks++;
            st.busy_s += now() - tb;
            std::vector<SrvJob*> keep;
            size_t ri = 0;
            for (SrvJob* j : active) {
                const bool ran = ri < run.size() && run[ri] == j;
                const int f = ran ? fate[ri++] : 0;
                if (f == 4) releaseSlots(j);
                if (f >= 1 && f <= 3) {
                    releaseSlots(j);
                    publish(j);
                    continue;
                }
                keep.push_back(j);
            }
            active.swap(keep);
            cvDone.notify_all();
        }
    }
};

}  // namespace

struct mc_server_s {
    std::unique_ptr<ServerBase> impl;
};

// ====================================================== no-allocation solve
// The one device array behind mc_solve_noalloc. Host code must not pass
// its name to a kernel (on the host it is only a stand-in for the symbol):
// noallocScratch() asks the runtime for its device address on the current
// device and the kernels receive that.
static __device__ __align__(256) unsigned char g_noallocScratch[MC_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noallocMu;
void* g_noallocPtr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noallocScratch on the current device, looked up once
// per device (the lookup can load this file's device code on that device).
int noallocScratch(void** out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return fail(MC_ERR_UNSUPPORTED, "mc_solve_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_noallocMu);
    if (!g_noallocPtr[dev]) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noallocScratch));
        if (!p) return fail(MC_ERR_CUDA, "mc_solve_noalloc: no device address for the scratch array");
        g_noallocPtr[dev] = p;
    }
    *out = g_noallocPtr[dev];
    return MC_OK;
}

// setupSession's buffers placed in `base` (cap bytes) instead of allocated:
// material tables, subdomain images, emitters, one half of the phonon state
// (the in-place dynamic schedule without compaction never touches the
// other), counters, status word, tally and checksum. The size check comes
// before any copy. Counters, status, tally and checksum are cleared by
// emitT; everything else is written here or by the emission kernel.
template <typename R>
int placeSession(mc_session_s* S, char* base, size_t cap) {
    const mc_material_s& m = *S->mat;
    const mc_domain_s& D = *S->dom;
    using V4 = typename Vec4<R>::T;
    // phonon allocation (montecarlo/problem.cpp:315-342), as in uploadDomain
    const long ne = (long)D.em.size();
    if (ne == 0) return fail(MC_ERR_ARG, "No phonons to emit");
    double wsum = 0.;
    for (double w : D.emWeight) wsum += w;
    std::vector<long long> cdf(ne);
    long long tot = 0;
    for (long i = 0; i < ne; ++i) {
        if (!(D.emWeight[i] > 0.)) return fail(MC_ERR_ARG, "No phonons to emit");
        const double rounded = std::ceil(D.emWeight[i] / wsum * S->desc.nemit - 0.5);
        tot += std::max(1LL, (long long)rounded);
        cdf[i] = tot;
    }
    S->nemit = (long)tot;
    S->power = wsum / (double)tot * m.fluxSum / 4.;
    S->rows = (int)problemRows(S->desc.problem, S->desc.cum_size);
    const size_t nt = (size_t)m.nw * m.np, n = (size_t)S->nemit;
    const size_t nval = (size_t)S->rows * std::max(D.cols, 1L);
    size_t off = 0;
    auto take = [&off](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t oVel = take(sizeof(R) * nt);
    const size_t oVt = take(sizeof(R) * nt);
    const size_t oWthr = take(8 * (size_t)m.nw);
    const size_t oPthr = take(8 * nt);
    const size_t oFwthr = take(8 * (size_t)m.nw);
    const size_t oFpthr = take(8 * nt);
    const size_t oGuide = take(2 * GUIDE);
    const size_t oSd = take(sizeof(SdomD<R>) * D.sd.size());
    const size_t oEm = take(sizeof(EmitterD) * ne);
    const size_t oCdf = take(sizeof(long long) * ne);
    const size_t oP0 = take(sizeof(V4) * n);
    const size_t oP1 = take(sizeof(V4) * n);
    const size_t oP2 = take(sizeof(uint4) * n);
    const size_t oCnt = take(sizeof(unsigned long long) * (C_NCOUNTERS + 5));
    const size_t oStatus = take(sizeof(unsigned int));
    const size_t oTally = take(sizeof(double) * nval);
    const size_t oCsum = take(sizeof(double) * 4);
    if (off > cap) {
        char msg[320];
        std::snprintf(msg, sizeof msg,
                      "mc_solve_noalloc: this problem needs %zu bytes of device scratch (%ld phonons x %zu B, "
                      "tables, %zu tally values), above the fixed maximum MC_NOALLOC_SCRATCH_BYTES = %zu; "
                      "use mc_solve or fewer phonons", off, S->nemit, 2 * sizeof(V4) + sizeof(uint4), nval, cap);
        return fail(MC_ERR_ARG, msg);
    }
    cudaStream_t s = S->stream;
    Params<R> P{};
    // material tables in the flight precision (as uploadMaterial)
    std::vector<R> vel(nt), vt(nt);
    double vmax = 0.;
    for (size_t i = 0; i < nt; ++i) {
        vel[i] = (R)m.vel[i];
        vt[i] = (R)(m.vel[i] * m.tau[i]);
        vmax = std::max(vmax, m.vel[i]);
    }
    S->vmax = vmax;
    std::vector<uint16_t> guide(GUIDE);
    for (int k = 0; k < GUIDE; ++k) {
        const unsigned long long x = (unsigned long long)k << (32 - GUIDE_BITS);
        long i = 0;
        while (i < m.nw - 1 && x >= m.swthr[i]) ++i;
        guide[k] = (uint16_t)i;
    }
    std::vector<SdomD<R>> sd(D.sd.size());
    for (size_t i = 0; i < sd.size(); ++i) castSdom(D.sd[i], sd[i], sizeof(R) == 4);
    CK(cudaMemcpyAsync(base + oVel, vel.data(), sizeof(R) * nt, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oVt, vt.data(), sizeof(R) * nt, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oWthr, m.swthr.data(), 8 * m.nw, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oPthr, m.spthr.data(), 8 * nt, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oFwthr, m.fwthr.data(), 8 * m.nw, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oFpthr, m.fpthr.data(), 8 * nt, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oGuide, guide.data(), 2 * GUIDE, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oSd, sd.data(), sizeof(SdomD<R>) * sd.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oEm, D.em.data(), sizeof(EmitterD) * ne, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + oCdf, cdf.data(), sizeof(long long) * ne, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the host vectors above end with this function
    P.vel = (const R*)(base + oVel);
    P.vt = (const R*)(base + oVt);
    P.wthr = (const unsigned long long*)(base + oWthr);
    P.pthr = (const unsigned long long*)(base + oPthr);
    P.fwthr = (const unsigned long long*)(base + oFwthr);
    P.fpthr = (const unsigned long long*)(base + oFpthr);
    P.wguide = (const uint16_t*)(base + oGuide);
    P.nw = (int)m.nw;
    P.np = (int)m.np;
    P.sd = (const SdomD<R>*)(base + oSd);
    P.nsd = (int)D.sd.size();
    P.em = (const EmitterD*)(base + oEm);
    P.emitCdf = (const long long*)(base + oCdf);
    P.nem = (int)ne;
    // one state half: P*out alias P*in
    P.P0in = P.P0out = (V4*)(base + oP0);
    P.P1in = P.P1out = (V4*)(base + oP1);
    P.P2in = P.P2out = (uint4*)(base + oP2);
    S->cnt_d = (unsigned long long*)(base + oCnt);
    S->status_d = (unsigned int*)(base + oStatus);
    S->tally_d = (double*)(base + oTally);
    S->csum_d = (double*)(base + oCsum);
    P.problem = S->desc.problem; P.rows = S->rows; P.cols = (int)D.cols;
    P.cumStep = cumStepOf(S->desc.problem, S->desc.maxscat, S->desc.cum_size);
    P.nemit = S->nemit;
    P.maxscat = S->desc.maxscat;
    P.maxloop = S->maxloop;
    P.dt = (R)S->desc.dt;
    P.nsteps = (int)S->desc.nsteps;
    P.ksteps = S->desc.steps_per_launch;
    P.key0 = (uint32_t)S->desc.seed;
    P.key1 = (uint32_t)(S->desc.seed >> 32);
    P.counters = S->cnt_d;
    P.qglobal = MC_DYN_GLOBAL_QUEUE ? S->cnt_d + C_NCOUNTERS + 4 : nullptr;
    P.cap = (unsigned long long)S->nemit;
    P.status = S->status_d;
    P.tally = S->tally_d;
    P.csum = S->csum_d;
    // launch configuration (as setupSession)
    const size_t tallyB = smemTallyBytes(S->rows, (int)D.cols);
    S->tm = S->desc.tally_mode;
    if (S->tm == MC_TALLY_AUTO) S->tm = tallyB <= 32 * 1024 ? TM_SHARED : TM_GLOBAL;
    {
        const SmemLayout L = singleLayout<R>((int)m.nw, (int)m.np, (int)D.sd.size(), S->rows, (int)D.cols,
                                             S->tm == TM_SHARED);
        S->smem = L.total;
        setSingleLayout(P, L);
    }
    if (S->smem > 227 * 1024) return fail(MC_ERR_UNSUPPORTED, "shared-memory tables exceed 227 KB");
    S->block = S->desc.block_size > 0 ? S->desc.block_size : 256;
    if (S->block % 32 || S->block > 256) return fail(MC_ERR_ARG, "block_size must be a multiple of 32, <= 256");
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const bool gen = D.needGen;
    S->gen = gen;
    const int occ = advanceOccupancy<R>(true, false, false, S->tm, gen, S->block, S->smem);
    if (occ <= 0) return fail(MC_ERR_UNSUPPORTED, "advance kernel cannot launch with this configuration");
    S->grid = S->desc.grid_blocks > 0 ? S->desc.grid_blocks : occ * nsm;
    paramsOf<R>(S) = P;
    return MC_OK;
}

}  // namespace

// ================================================================== C ABI
extern "C" {

const char* mc_last_error(void) { return g_err.c_str(); }
const char* mc_version(void) { return "montecarlocpp_gb300 0.1 (sm_103a)"; }

int mc_material_create(const double* disp, long nw, long np, const double* relax, double T, mc_material_h* out) {
    if (!out) return fail(MC_ERR_ARG, "null output handle");
    return buildMaterial(disp, nw, np, relax, T, out);
}

int mc_material_load(const char* dp, const char* rp, double T, mc_material_h* out) {
    if (!dp || !rp || !out) return fail(MC_ERR_ARG, "null argument");
    std::vector<double> a, b;
    if (!readAll(dp, a)) return fail(MC_ERR_IO, "Error opening dispersion file");
    if (!readAll(rp, b)) return fail(MC_ERR_IO, "Error opening relaxation time file");
    if (a.size() < 2) return fail(MC_ERR_ARG, "Invalid dispersion file");
    long nw = (long)a[0], np = (long)a[1];
    if (nw <= 0 || np <= 0) return fail(MC_ERR_ARG, "Invalid dispersion file");
    if ((long)a.size() < 2 + nw * (2 + 2 * np) || (long)b.size() < 8 * np)
        return fail(MC_ERR_ARG, "Array extraction failed");
    return buildMaterial(a.data() + 2, nw, np, b.data(), T, out);
}

int mc_material_create_many(const double* disp, long nw, long np, const double* relax, const double* T, int n,
                            mc_material_h* out) {
    if (!disp || !relax || !T || !out || n <= 0 || nw <= 0 || np <= 0 || np > 255 || nw > 65535)
        return fail(MC_ERR_ARG, "invalid arguments");
    for (int t = 0; t < n; ++t)
        if (!(T[t] > 0.)) return fail(MC_ERR_ARG, "temperature must be positive");
    for (long p = 0; p < np; ++p)
        for (int j = 0; j < 2; ++j)
            if (relax[p * 8 + 4 * j] < 0.) return fail(MC_ERR_ARG, "Scattering times cannot be negative");
    int rc = ensureDevice();
    if (rc) return rc;
    const long nt = nw * np, nc = 2 + 2 * np;
    std::vector<double> omega(nw), domega(nw), vel(nt), dos(nt);
    for (long w = 0; w < nw; ++w) {
        omega[w] = disp[w * nc];
        domega[w] = disp[w * nc + 1];
        for (long p = 0; p < np; ++p) {
            vel[w * np + p] = disp[w * nc + 2 + 2 * p];
            dos[w * np + p] = disp[w * nc + 3 + 2 * p];
        }
    }
    // one device allocation: inputs, then per temperature the outputs and
    // the pdf scratch
    const size_t nIn = 2 * (size_t)nw + 2 * (size_t)nt + 8 * (size_t)np + (size_t)n;
    const size_t nD = (size_t)n * ((size_t)nt + 4 + 3 * (size_t)nt + 2 * (size_t)nw);
    const size_t nU = (size_t)n * (2 * (size_t)nw + 2 * (size_t)nt);
    void* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, sizeof(double) * (nIn + nD) + sizeof(unsigned long long) * nU + sizeof(int) * n);
    if (e != cudaSuccess) return cudaFail(e, "cudaMalloc");
    std::unique_ptr<void, void (*)(void*)> hold(buf, [](void* q) { cudaFree(q); });
    MatBuildArgs A;
    A.nw = nw; A.np = np;
    double* in = (double*)buf;
    A.omega = in; in += nw;
    A.domega = in; in += nw;
    A.vel = in; in += nt;
    A.dos = in; in += nt;
    A.relax = in; in += 8 * np;
    A.T = in; in += n;
    A.tau = in; in += (size_t)n * nt;
    A.sums = in; in += (size_t)n * 4;
    A.scratch = in; in += (size_t)n * 3 * nt;
    A.rows = in; in += (size_t)n * 2 * nw;
    unsigned long long* u = (unsigned long long*)in;
    A.swthr = u; u += (size_t)n * nw;
    A.fwthr = u; u += (size_t)n * nw;
    A.spthr = u; u += (size_t)n * nt;
    A.fpthr = u; u += (size_t)n * nt;
    A.status = (int*)u;
    CK(cudaMemcpy((void*)A.omega, omega.data(), sizeof(double) * nw, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void*)A.domega, domega.data(), sizeof(double) * nw, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void*)A.vel, vel.data(), sizeof(double) * nt, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void*)A.dos, dos.data(), sizeof(double) * nt, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void*)A.relax, relax, sizeof(double) * 8 * np, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((void*)A.T, T, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(launchBuildMaterials(A, n, nullptr));
    std::vector<double> tau((size_t)n * nt), sums((size_t)n * 4);
    std::vector<unsigned long long> thr(nU);
    std::vector<int> status(n);
    CK(cudaMemcpy(tau.data(), A.tau, sizeof(double) * tau.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(sums.data(), A.sums, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(thr.data(), A.swthr, sizeof(unsigned long long) * nU, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(status.data(), A.status, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int t = 0; t < n; ++t) {
        if (status[t]) return fail(MC_ERR_ARG, "Scattering time model produced infinite values or a velocity is zero");
        if (!(sums[4 * t + 1] > 0.) || !(sums[4 * t + 2] > 0.)) return fail(MC_ERR_ARG, "material has no phonons to draw");
    }
    for (int t = 0; t < n; ++t) {
        mc_material_s* m = new mc_material_s;
        m->nw = nw; m->np = np; m->T = T[t];
        m->omega = omega;
        m->vel = vel;
        m->tau.assign(tau.begin() + (size_t)t * nt, tau.begin() + (size_t)(t + 1) * nt);
        m->energySum = sums[4 * t]; m->fluxSum = sums[4 * t + 1]; m->scatSum = sums[4 * t + 2];
        m->cond = sums[4 * t + 3];
        const unsigned long long* sw = thr.data() + (size_t)t * nw;
        const unsigned long long* fw = thr.data() + (size_t)n * nw + (size_t)t * nw;
        const unsigned long long* sp = thr.data() + 2 * (size_t)n * nw + (size_t)t * nt;
        const unsigned long long* fp = thr.data() + 2 * (size_t)n * nw + (size_t)n * nt + (size_t)t * nt;
        m->swthr.assign(sw, sw + nw);
        m->fwthr.assign(fw, fw + nw);
        m->spthr.assign(sp, sp + nt);
        m->fpthr.assign(fp, fp + nt);
        out[t] = m;
    }
    return MC_OK;
}

int mc_material_thresholds(mc_material_h m, uint64_t* swthr, uint64_t* spthr, uint64_t* fwthr, uint64_t* fpthr) {
    if (!m) return fail(MC_ERR_ARG, "null argument");
    const size_t nw = (size_t)m->nw, nt = (size_t)m->nw * m->np;
    if (swthr) std::memcpy(swthr, m->swthr.data(), 8 * nw);
    if (spthr) std::memcpy(spthr, m->spthr.data(), 8 * nt);
    if (fwthr) std::memcpy(fwthr, m->fwthr.data(), 8 * nw);
    if (fpthr) std::memcpy(fpthr, m->fpthr.data(), 8 * nt);
    return MC_OK;
}

int mc_material_sums(mc_material_h m, double out[4]) {
    if (!m || !out) return fail(MC_ERR_ARG, "null argument");
    out[0] = m->energySum; out[1] = m->fluxSum; out[2] = m->scatSum; out[3] = m->cond;
    return MC_OK;
}

int mc_material_tables(mc_material_h m, double* vel, double* tau) {
    if (!m) return fail(MC_ERR_ARG, "null argument");
    if (vel) std::memcpy(vel, m->vel.data(), sizeof(double) * m->vel.size());
    if (tau) std::memcpy(tau, m->tau.data(), sizeof(double) * m->tau.size());
    return MC_OK;
}

void mc_material_destroy(mc_material_h m) { delete m; }

int mc_domain_create(const mc_pped_desc* ps, int n, const mc_pair_desc* qs, int nq, mc_domain_h* out) {
    if (!out) return fail(MC_ERR_ARG, "null output handle");
    if (nq > 0 && !qs) return fail(MC_ERR_ARG, "null pair list");
    if (!ps || n <= 0) return fail(MC_ERR_ARG, "Domain setup not complete");
    std::vector<mc_sdom_desc> v;
    for (int i = 0; i < n; ++i) v.push_back(sdomOfPped(ps[i]));
    return buildDomain(v.data(), n, qs, nq, out);
}

int mc_domain_create_shapes(const mc_sdom_desc* ps, int n, const mc_pair_desc* qs, int nq, mc_domain_h* out) {
    if (!out) return fail(MC_ERR_ARG, "null output handle");
    if (nq > 0 && !qs) return fail(MC_ERR_ARG, "null pair list");
    return buildDomain(ps, n, qs, nq, out);
}

long mc_domain_cols(mc_domain_h d) { return d ? d->cols : -1; }

int mc_domain_cell_volumes(mc_domain_h d, double* out) {
    if (!d || !out) return fail(MC_ERR_ARG, "null argument");
    std::memcpy(out, d->cellVol.data(), sizeof(double) * d->cellVol.size());
    return MC_OK;
}

void mc_domain_destroy(mc_domain_h d) { delete d; }

int mc_session_create(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, mc_session_h* out) {
    if (!m || !d || !p || !out) return fail(MC_ERR_ARG, "null argument");
    if (int rcp = checkProblem(*p)) return rcp;
    if (p->nemit <= 0 || p->maxscat <= 0 || p->maxloop < 0) return fail(MC_ERR_ARG, "Invalid problem arguments");
    if (!(p->dt > 0.) || p->nsteps <= 0 || p->nsteps > (1L << 30)) return fail(MC_ERR_ARG, "dt and nsteps must be positive");
    if (p->steps_per_launch <= 0) return fail(MC_ERR_ARG, "steps_per_launch must be >= 1");
    if (p->precision != 32 && p->precision != 64) return fail(MC_ERR_ARG, "precision must be 32 or 64");
    if ((p->replay_words == nullptr) != (p->replay_offsets == nullptr)) return fail(MC_ERR_ARG, "replay needs words and offsets");
    if (p->log && (p->log_cap <= 0 || p->log_phonons <= 0 || !p->log_counts)) return fail(MC_ERR_ARG, "invalid log request");
    int rc = ensureDevice();
    if (rc) return rc;
    mc_session_s* S = new mc_session_s;
    S->mat = m; S->dom = d; S->desc = *p;
    S->prec = p->precision;
    S->replay = p->replay_words != nullptr;
    S->logging = p->log != nullptr;
    if (p->schedule < MC_SCHED_AUTO || p->schedule > MC_SCHED_DYNAMIC) { delete S; return fail(MC_ERR_ARG, "invalid schedule"); }
    S->dyn = p->schedule == MC_SCHED_DYNAMIC || (p->schedule == MC_SCHED_AUTO && p->steps_per_launch > 1);
    S->maxloop = p->maxloop != 0 ? p->maxloop : 100 * p->maxscat;
    if (p->stream) S->stream = (cudaStream_t)p->stream;
    else {
        cudaError_t e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete S; return cudaFail(e, "cudaStreamCreate"); }
        S->ownStream = true;
    }
    rc = S->prec == 32 ? setupSession<float>(S) : setupSession<double>(S);
    if (rc) { std::string msg = g_err; freeSession(S); g_err = msg; return rc; }
    *out = S;
    return MC_OK;
}

int mc_session_emit(mc_session_h s) {
    if (!s) return fail(MC_ERR_ARG, "null session");
    s->parity = 0;
    return s->prec == 32 ? emitT<float>(s) : emitT<double>(s);
}

int mc_session_advance(mc_session_h s, int nl, int* done) {
    if (!s || nl < 0) return fail(MC_ERR_ARG, "invalid argument");
    return s->prec == 32 ? advanceT<float>(s, nl, done) : advanceT<double>(s, nl, done);
}

int mc_session_result(mc_session_h s, double* out, mc_stats* st) {
    if (!s) return fail(MC_ERR_ARG, "null session");
    return resultImpl(s, out, st);
}

size_t mc_session_state_bytes(mc_session_h s) { return s ? s->stateBytes : 0; }

// ---------------------------------------------------------------- snapshot
// A session's resumable state, in one host buffer: a header that must match
// the restoring session, then the live half of the phonon state, the live
// counts (block regions of both halves in the static schedule; the slot
// count in the dynamic one sits among the counters), counters, status,
// raw field, checksums and, in replay mode, the per-phonon stream cursors.
// Philox streams are keyed by phonon id and event index, so a restored
// session continues every trajectory exactly.
namespace {
struct SnapHeader {
    uint32_t magic, version;
    int32_t prec, dyn, grid, block, rows, replay;
    int64_t nemit, slots, cols;
    int32_t step, parity, launches, sinceCompact;
    // the problem the state belongs to: a session that differs in any of
    // these would continue on another Philox key, window or stop rule
    int32_t problem, stepsPerLaunch;
    int64_t nsteps, maxscat, maxloop, cumSize;
    uint64_t seed;
    double dt;
};
constexpr uint32_t SNAP_MAGIC = 0x5353434Du;  // "MCSS"
constexpr uint32_t SNAP_VERSION = 2;

struct SnapPart { void* dev; size_t bytes; };

std::vector<SnapPart> snapParts(mc_session_s* S) {
    std::vector<SnapPart> v;
    const size_t v4 = S->prec == 32 ? sizeof(float4) : sizeof(dbl4);
    const int half = S->parity;
    void *a, *b, *c;
    if (S->prec == 32) {
        const Params<float>& P = S->p32;
        a = half ? (void*)P.P0out : (void*)P.P0in; b = half ? (void*)P.P1out : (void*)P.P1in;
        c = half ? (void*)P.P2out : (void*)P.P2in;
    } else {
        const Params<double>& P = S->p64;
        a = half ? (void*)P.P0out : (void*)P.P0in; b = half ? (void*)P.P1out : (void*)P.P1in;
        c = half ? (void*)P.P2out : (void*)P.P2in;
    }
    const size_t n = (size_t)S->slots;
    v.push_back({a, v4 * n});
    v.push_back({b, v4 * n});
    v.push_back({c, sizeof(uint4) * n});
    v.push_back({S->cnt_d, sizeof(unsigned long long) * (C_NCOUNTERS + 4)});
    v.push_back({S->status_d, sizeof(unsigned int)});
    v.push_back({S->tally_d, sizeof(double) * (size_t)S->rows * (size_t)std::max(S->dom->cols, 1L)});
    v.push_back({S->csum_d, sizeof(double) * 4});
    if (S->reg_d) v.push_back({S->reg_d, sizeof(unsigned) * 4 * (size_t)S->grid});
    if (S->replay) v.push_back({S->rcur_d, sizeof(uint32_t) * (size_t)S->nemit});
    return v;
}

SnapHeader snapHeader(const mc_session_s* S) {
    SnapHeader h;
    std::memset(&h, 0, sizeof(h));
    h.magic = SNAP_MAGIC; h.version = SNAP_VERSION;
    h.prec = S->prec; h.dyn = S->dyn ? 1 : 0; h.grid = S->grid; h.block = S->block; h.rows = S->rows;
    h.replay = S->replay ? 1 : 0;
    h.nemit = S->nemit; h.slots = S->slots; h.cols = S->dom->cols;
    h.step = S->step; h.parity = S->parity; h.launches = S->launches; h.sinceCompact = S->sinceCompact;
    h.problem = S->desc.problem; h.stepsPerLaunch = S->desc.steps_per_launch;
    h.nsteps = S->desc.nsteps; h.maxscat = S->desc.maxscat; h.maxloop = S->maxloop; h.cumSize = S->desc.cum_size;
    h.seed = S->desc.seed; h.dt = S->desc.dt;
    return h;
}
}  // namespace

size_t mc_session_snapshot_bytes(mc_session_h s) {
    if (!s) return 0;
    size_t n = sizeof(SnapHeader);
    for (const SnapPart& p : snapParts(s)) n += (p.bytes + 7) & ~(size_t)7;
    return n;
}

int mc_session_snapshot(mc_session_h s, void* buf, size_t bytes) {
    if (!s || !buf) return fail(MC_ERR_ARG, "null argument");
    if (s->logging) return fail(MC_ERR_UNSUPPORTED, "sessions that log trajectories cannot be snapshotted");
    if (bytes < mc_session_snapshot_bytes(s)) return fail(MC_ERR_ARG, "snapshot buffer too small");
    CK(cudaStreamSynchronize(s->stream));
    char* p = (char*)buf;
    const SnapHeader h = snapHeader(s);
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    for (const SnapPart& q : snapParts(s)) {
        CK(cudaMemcpy(p, q.dev, q.bytes, cudaMemcpyDeviceToHost));
        p += (q.bytes + 7) & ~(size_t)7;
    }
    return MC_OK;
}

int mc_session_restore(mc_session_h s, const void* buf, size_t bytes) {
    if (!s || !buf) return fail(MC_ERR_ARG, "null argument");
    if (s->logging) return fail(MC_ERR_UNSUPPORTED, "sessions that log trajectories cannot be restored");
    if (bytes < sizeof(SnapHeader)) return fail(MC_ERR_ARG, "snapshot buffer too small");
    SnapHeader h;
    std::memcpy(&h, buf, sizeof(h));
    const SnapHeader mine = snapHeader(s);
    if (h.magic != SNAP_MAGIC || h.version != SNAP_VERSION) return fail(MC_ERR_ARG, "not a session snapshot");
    if (h.prec != mine.prec || h.dyn != mine.dyn || h.grid != mine.grid || h.block != mine.block ||
        h.rows != mine.rows || h.replay != mine.replay || h.nemit != mine.nemit || h.slots != mine.slots ||
        h.cols != mine.cols)
        return fail(MC_ERR_ARG, "snapshot of a different problem or launch configuration");
    if (h.problem != mine.problem || h.stepsPerLaunch != mine.stepsPerLaunch || h.nsteps != mine.nsteps ||
        h.maxscat != mine.maxscat || h.maxloop != mine.maxloop || h.cumSize != mine.cumSize || h.seed != mine.seed ||
        h.dt != mine.dt)
        return fail(MC_ERR_ARG, "snapshot of a session with another seed, time step, horizon, window or problem");
    if (h.step < 0 || h.step > (int)s->desc.nsteps || (h.parity != 0 && h.parity != 1))
        return fail(MC_ERR_ARG, "corrupt snapshot header");
    // the parts' sizes follow from the fields compared above, so the whole
    // buffer is checked before anything of the session changes
    if (bytes < mc_session_snapshot_bytes(s)) return fail(MC_ERR_ARG, "snapshot buffer too small");
    CK(cudaStreamSynchronize(s->stream));
    s->step = h.step; s->parity = h.parity; s->launches = h.launches; s->sinceCompact = h.sinceCompact;
    const char* p = (const char*)buf + sizeof(h);
    for (const SnapPart& q : snapParts(s)) {
        CK(cudaMemcpy(q.dev, p, q.bytes, cudaMemcpyHostToDevice));
        p += (q.bytes + 7) & ~(size_t)7;
    }
    return MC_OK;
}

void mc_session_destroy(mc_session_h s) { freeSession(s); }

int mc_solve(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, double* out, mc_stats* st) {
    mc_session_h s = nullptr;
    int rc = mc_session_create(m, d, p, &s);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s->stream);
    rc = mc_session_emit(s);
    int done = 0;
    while (!rc && !done) rc = mc_session_advance(s, 64, &done);
    cudaEventRecord(e1, s->stream);
    if (!rc) rc = mc_session_result(s, out, st);
    float ms = 0.f;
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (st) st->kernel_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::string msg = g_err;
    mc_session_destroy(s);
    g_err = msg;
    return rc;
}

// Bounded-wait self-check: a wait that nothing completes must give up with
// S_TIMEOUT after about limit_ms, and the device must stay usable.
int mc_check_bounded_wait(double limit_ms, unsigned* status, double* waited_ms) {
    if (!(limit_ms > 0.) || limit_ms > 1000.) return fail(MC_ERR_ARG, "limit_ms must be in (0, 1000]");
    int rc = ensureDevice();
    if (rc) return rc;
    unsigned* st_d = nullptr;
    unsigned long long* w_d = nullptr;
    CK(cudaMalloc(&st_d, sizeof(unsigned)));
    CK(cudaMalloc(&w_d, sizeof(unsigned long long)));
    CK(cudaMemset(st_d, 0, sizeof(unsigned)));
    cudaError_t e = launchWaitCheck(st_d, (unsigned long long)(limit_ms * 1e6), w_d, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    unsigned st = 0;
    unsigned long long w = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, st_d, sizeof(st), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&w, w_d, sizeof(w), cudaMemcpyDeviceToHost);
    cudaFree(st_d);
    cudaFree(w_d);
    if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("bounded-wait check: ") + cudaGetErrorString(e));
    if (status) *status = st;
    if (waited_ms) *waited_ms = (double)w * 1e-6;
    return MC_OK;
}

// Replicas (montecarlo/main.cpp:181-210): nsim solves of one session whose
// Philox key is seed + i for replica i, folded into Statistics' Welford
// mean and sum of squared deviations (montecarlo/field.cpp:226-262).
int mc_solve_replicas(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, long nsim, double* mean, double* sd,
                      mc_stats* st) {
    if (!m || !d || !p || !mean || nsim < 1) return fail(MC_ERR_ARG, "mc_solve_replicas: null argument or nsim < 1");
    if (p->replay_words || p->replay_offsets || p->log)
        return fail(MC_ERR_UNSUPPORTED, "mc_solve_replicas: replicas take neither replay streams nor logs");
    mc_session_h s = nullptr;
    int rc = mc_session_create(m, d, p, &s);
    if (rc) return rc;
    const size_t nval = (size_t)s->rows * (size_t)s->dom->cols;
    std::vector<double> x(nval), mu(nval, 0.), m2(nval, 0.);
    mc_stats tot;
    std::memset(&tot, 0, sizeof(tot));
    for (long i = 0; i < nsim && !rc; ++i) {
        const uint64_t seed = p->seed + (uint64_t)i;
        s->desc.seed = seed;
        s->p32.key0 = s->p64.key0 = (uint32_t)seed;
        s->p32.key1 = s->p64.key1 = (uint32_t)(seed >> 32);
        rc = mc_session_emit(s);
        int done = 0;
        while (!rc && !done) rc = mc_session_advance(s, 64, &done);
        mc_stats one;
        if (!rc) rc = mc_session_result(s, x.data(), &one);
        if (rc) break;
        // Statistics::add
        const double n = (double)(i + 1);
        for (size_t k = 0; k < nval; ++k) {
            const double dl = x[k] - mu[k];
            mu[k] += dl / n;
            m2[k] += dl * (x[k] - mu[k]);
        }
        if (i == 0) tot = one;
        else {
            tot.phonon_steps += one.phonon_steps; tot.events += one.events; tot.scatters += one.scatters;
            tot.escapes += one.escapes; tot.horizon_stops += one.horizon_stops; tot.maxscat_stops += one.maxscat_stops;
            tot.maxloop_stops += one.maxloop_stops; tot.absorbed += one.absorbed; tot.nonfinite += one.nonfinite;
            tot.status |= one.status; tot.launches += one.launches;
            for (int r = 0; r < 4; ++r) tot.checksum[r] += one.checksum[r];
        }
    }
    if (!rc) {
        std::memcpy(mean, mu.data(), sizeof(double) * nval);
        // Statistics::variance: s / (n - 1), zero below two replicas
        if (sd)
            for (size_t k = 0; k < nval; ++k) sd[k] = nsim < 2 ? 0. : std::sqrt(m2[k] / (double)(nsim - 1));
        if (st) *st = tot;
    }
    std::string msg = g_err;
    mc_session_destroy(s);
    g_err = msg;
    return rc;
}

// The solve of mc_solve with every device buffer inside g_noallocScratch:
// a session object on the host stack whose pointers lead into the array,
// driven through the same emission, advance and result steps. Nothing is
// allocated on the device and nothing is freed.
int mc_solve_noalloc(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, double* out, mc_stats* st) {
    if (!m || !d || !p) return fail(MC_ERR_ARG, "null argument");
    if (int rcp = checkProblem(*p)) return rcp;
    if (p->nemit <= 0 || p->maxscat <= 0 || p->maxloop < 0) return fail(MC_ERR_ARG, "Invalid problem arguments");
    if (!(p->dt > 0.) || p->nsteps <= 0 || p->nsteps > (1L << 30)) return fail(MC_ERR_ARG, "dt and nsteps must be positive");
    if (p->steps_per_launch <= 0) return fail(MC_ERR_ARG, "steps_per_launch must be >= 1");
    if (p->precision != 32 && p->precision != 64) return fail(MC_ERR_ARG, "precision must be 32 or 64");
    if (p->replay_words || p->replay_offsets || p->log)
        return fail(MC_ERR_UNSUPPORTED, "mc_solve_noalloc: replay streams and trajectory logs are not supported; use mc_solve");
    // the descriptor is validated as mc_solve validates it, although the
    // in-place dynamic schedule always runs here
    if (p->schedule < MC_SCHED_AUTO || p->schedule > MC_SCHED_DYNAMIC) return fail(MC_ERR_ARG, "invalid schedule");
    if (p->compact_interval < 0) return fail(MC_ERR_ARG, "compact_interval must be >= 0");
    int rc = ensureDevice();
    if (rc) return rc;
    void* scratch = nullptr;
    rc = noallocScratch(&scratch);
    if (rc) return rc;
    mc_session_s S;
    S.mat = m; S.dom = d; S.desc = *p;
    S.desc.schedule = MC_SCHED_DYNAMIC;
    S.desc.compact_interval = 0;
    S.prec = p->precision;
    S.dyn = true;
    S.maxloop = p->maxloop != 0 ? p->maxloop : 100 * p->maxscat;
    S.stream = (cudaStream_t)p->stream;
    const bool f32 = S.prec == 32;
    rc = f32 ? placeSession<float>(&S, (char*)scratch, MC_NOALLOC_SCRATCH_BYTES)
             : placeSession<double>(&S, (char*)scratch, MC_NOALLOC_SCRATCH_BYTES);
    if (!rc) rc = f32 ? emitT<float>(&S) : emitT<double>(&S);
    int done = 0;
    while (!rc && !done) rc = f32 ? advanceT<float>(&S, 64, &done) : advanceT<double>(&S, 64, &done);
    if (!rc) return resultImpl(&S, out, st);
    // no launch of this call may still write the array after it returns
    std::string msg = g_err;
    cudaStreamSynchronize(S.stream);
    g_err = msg;
    return rc;
}


int mc_batch_create(int n, const mc_material_h* mats, const mc_domain_h* doms, const mc_problem_desc* probs,
                    const mc_batch_desc* bd, mc_batch_h* out) {
    if (n <= 0 || !mats || !doms || !probs || !bd || !out) return fail(MC_ERR_ARG, "invalid batch arguments");
    for (int i = 0; i < n; ++i)
        if (!mats[i] || !doms[i]) return fail(MC_ERR_ARG, "null material or domain in batch");
    if (!(bd->dt > 0.) || bd->nsteps <= 0 || bd->nsteps > (1L << 30)) return fail(MC_ERR_ARG, "dt and nsteps must be positive");
    if (bd->precision != 32 && bd->precision != 64) return fail(MC_ERR_ARG, "precision must be 32 or 64");
    if (bd->steps_per_launch < 0) return fail(MC_ERR_ARG, "steps_per_launch must be >= 0");
    int rc = ensureDevice();
    if (rc) return rc;
    mc_batch_s* B = new mc_batch_s;
    B->n = n;
    B->prec = bd->precision;
    B->bd = *bd;
    B->mats.assign(mats, mats + n);
    B->doms.assign(doms, doms + n);
    B->probs.assign(probs, probs + n);
    if (bd->stream) B->stream = (cudaStream_t)bd->stream;
    else {
        cudaError_t e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete B; return cudaFail(e, "cudaStreamCreate"); }
        B->ownStream = true;
    }
    rc = B->prec == 32 ? setupBatch<float>(B) : setupBatch<double>(B);
    if (rc) { std::string msg = g_err; freeBatch(B); g_err = msg; return rc; }
    *out = B;
    return MC_OK;
}

int mc_batch_run(mc_batch_h b) {
    if (!b) return fail(MC_ERR_ARG, "null batch");
    return b->prec == 32 ? runBatch<float>(b) : runBatch<double>(b);
}

int mc_batch_result(mc_batch_h b, int i, double* out, mc_stats* st) {
    if (!b || i < 0 || i >= b->n) return fail(MC_ERR_ARG, "invalid batch instance");
    CK(cudaStreamSynchronize(b->stream));
    const int rows = b->rows[i], cols = b->cols[i];
    std::vector<double> f((size_t)rows * cols + (size_t)rows * (cols + 1) + 4);
    CK(cudaMemcpy(f.data(), b->fields + b->fieldOff[i], sizeof(double) * f.size(), cudaMemcpyDeviceToHost));
    const mc_material_s& m = *b->mats[i];
    const mc_domain_s& D = *b->doms[i];
    const int problem = b->probs[i].problem;
    if (out) {
        std::vector<double> v(f.begin(), f.begin() + (size_t)rows * cols);
        postProcess(problem, rows, cols, m.energySum, v.data());
        for (int c = 0; c < cols; ++c)
            for (int r = 0; r < rows; ++r)
                out[(size_t)c * rows + r] = b->power[i] * (v[(size_t)c * rows + r] / D.cellVol[c]);
    }
    if (st) {
        int rc = batchCounters(b, st);
        st->nemit = b->nemit[i];
        st->power = b->power[i];
        st->rows = rows;
        st->cols = cols;
        const double* cs = f.data() + (size_t)rows * cols + (size_t)rows * (cols + 1);
        for (int r = 0; r < 4; ++r) st->checksum[r] = cs[r];
        return rc;
    }
    return MC_OK;
}

int mc_batch_stats(mc_batch_h b, mc_stats* st) {
    if (!b || !st) return fail(MC_ERR_ARG, "null argument");
    return batchCounters(b, st);
}

size_t mc_batch_state_bytes(mc_batch_h b) { return b ? b->stateBytes : 0; }

void mc_batch_destroy(mc_batch_h b) { freeBatch(b); }

int mc_server_create(const mc_server_desc* d, mc_server_h* out) {
    if (!d || !out) return fail(MC_ERR_ARG, "null argument");
    if (!(d->dt > 0.) || d->nsteps <= 0 || d->nsteps > (1L << 30)) return fail(MC_ERR_ARG, "dt and nsteps must be positive");
    if (d->precision != 32 && d->precision != 64) return fail(MC_ERR_ARG, "precision must be 32 or 64");
    if (d->groups < 2 || d->groups > MAX_GROUPS) return fail(MC_ERR_ARG, "groups must be in 2..8");
    if (d->max_active < 1 || d->max_active > 512) return fail(MC_ERR_ARG, "max_active must be in 1..512");
    if (!(d->target_rel_se > 0.) || d->max_rounds < 1 || d->min_rounds < 1) return fail(MC_ERR_ARG, "invalid stopping rule");
    if (d->steps_per_window < 0 || d->steps_per_window > d->nsteps ||
        (d->steps_per_window > 0 && d->nsteps % d->steps_per_window != 0))
        return fail(MC_ERR_ARG, "steps_per_window must be 0 or a divisor of nsteps");
    int rc = ensureDevice();
    if (rc) return rc;
    std::unique_ptr<ServerBase> impl;
    if (d->precision == 32) { auto* t = new ServerT<float>; t->d = *d; impl.reset(t); rc = t->init(); }
    else { auto* t = new ServerT<double>; t->d = *d; impl.reset(t); rc = t->init(); }
    if (rc) return rc;
    impl->t0 = Clock::now();
    ServerBase* b = impl.get();
    b->th = std::thread([b] { b->loop(); });
    *out = new mc_server_s{std::move(impl)};
    return MC_OK;
}

int mc_server_submit(mc_server_h s, const mc_request* r, long* ticket) {
    if (!s || !r || !ticket) return fail(MC_ERR_ARG, "null argument");
    if (!r->mat || !r->dom || r->nemit <= 0 || r->maxscat <= 0 || r->maxloop < 0 || r->axis < 0 || r->axis > 2 ||
        r->max_rounds < 0)
        return fail(MC_ERR_ARG, "invalid request");
    if (!std::isfinite(r->volume) || r->volume < 0. || !std::isfinite(r->gradient))
        return fail(MC_ERR_ARG, "request volume and gradient must be finite");
    if (r->problem != MC_FLUX && r->problem != MC_MULTI) return fail(MC_ERR_ARG, "kappa needs a flux problem");
    ServerBase* b = s->impl.get();
    SrvJob* j = new SrvJob;
    j->req = *r;
    std::lock_guard<std::mutex> lk(b->mu);
    j->ticket = b->nextTicket++;
    j->tSubmit = b->now();
    b->jobs[j->ticket] = j;
    b->pending.push_back(j);
    b->st.submitted++;
    *ticket = j->ticket;
    b->cv.notify_all();
    return MC_OK;
}

int mc_server_cancel(mc_server_h s, long ticket) {
    if (!s) return fail(MC_ERR_ARG, "null server");
    ServerBase* b = s->impl.get();
    std::lock_guard<std::mutex> lk(b->mu);
    auto it = b->jobs.find(ticket);
    if (it == b->jobs.end()) return fail(MC_ERR_ARG, "unknown ticket");
    SrvJob* j = it->second;
    if (j->done) return 0;
    auto q = std::find(b->pending.begin(), b->pending.end(), j);
    if (q != b->pending.end()) {
        // queued: nothing on the device yet
        b->pending.erase(q);
        j->status = MC_ERR_CANCELLED;
        j->tDone = b->now();
        j->done = true;
        b->st.completed++;
        b->cvDone.notify_all();
        return 1;
    }
    j->cancel = true;  // the loop drops it at the next window boundary
    b->cv.notify_all();
    return 1;
}

static int pollLocked(ServerBase* b, long ticket, mc_result* res, double* field) {
    auto it = b->jobs.find(ticket);
    if (it == b->jobs.end()) return fail(MC_ERR_ARG, "unknown ticket");
    SrvJob* j = it->second;
    if (!j->done) return 0;
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->kappa = j->kappa();
        res->kappa_se = j->dof > 0 ? j->se() : 0.;
        res->rounds = j->rounds;
        res->phonons = (long)j->sumN;
        res->phonon_steps = j->steps;
        res->t_submit = j->tSubmit;
        res->t_admit = j->tAdmit;
        res->t_done = j->tDone;
        res->status = j->status;
    }
    if (field && !j->field.empty()) std::memcpy(field, j->field.data(), sizeof(double) * j->field.size());
    return 1;
}

int mc_server_poll(mc_server_h s, long ticket, mc_result* res, double* field) {
    if (!s) return fail(MC_ERR_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->impl->mu);
    return pollLocked(s->impl.get(), ticket, res, field);
}

int mc_server_wait(mc_server_h s, long ticket, double timeout_s, mc_result* res, double* field) {
    if (!s) return fail(MC_ERR_ARG, "null server");
    ServerBase* b = s->impl.get();
    std::unique_lock<std::mutex> lk(b->mu);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    for (;;) {
        int rc = pollLocked(b, ticket, res, field);
        if (rc != 0) return rc;
        if (b->cvDone.wait_until(lk, until) == std::cv_status::timeout) return pollLocked(b, ticket, res, field);
    }
}

int mc_server_stats(mc_server_h s, mc_server_counters* st) {
    if (!s || !st) return fail(MC_ERR_ARG, "null argument");
    ServerBase* b = s->impl.get();
    std::lock_guard<std::mutex> lk(b->mu);
    *st = b->st;
    st->queued = (long)b->pending.size();
    st->active = (long)b->active.size();
    st->uptime_s = b->now();
    return MC_OK;
}

double mc_server_clock(mc_server_h s) { return s ? s->impl->now() : 0.; }

void mc_server_destroy(mc_server_h s) {
    if (!s) return;
    ServerBase* b = s->impl.get();
    {
        std::lock_guard<std::mutex> lk(b->mu);
        b->stop = true;
        b->cv.notify_all();
    }
    if (b->th.joinable()) b->th.join();
    for (auto& kv : b->jobs) { freeJobDevice(kv.second); delete kv.second; }
    delete s;
}

}  // extern "C"


