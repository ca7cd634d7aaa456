// mc_gb300.hpp -- C++ host mirror of montecarlocpp's Material / Domain /
// Problem API over the C ABI of mc_gb300.h (header only).
//
// Names, constructor arguments and meanings follow the reference:
//   Material(disp, relax, T)                  montecarlo/material.h:51-67
//   FilmDomain(dim, div, dT), BulkDomain(...)  montecarlo/domain.h:93-137
//   TempProblem / FluxProblem / MultiProblem
//       (mat, dom, nemit, maxscat, maxloop)   montecarlo/problem.h:157-203
//   CumTempProblem / CumFluxProblem (mat, dom, nemit, size, maxscat, maxloop)
//                                         montecarlo/problem.h:205-239
// FieldProblem::solve() returns the rows x cols field in the column-major
// layout of Eigen::ArrayXXd (montecarlo/problem.cpp:370-445); errors that the
// reference turns into BOOST_ASSERT_MSG aborts are thrown as mcgb::Error.
#ifndef MC_GB300_HPP
#define MC_GB300_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mc_gb300.h"

namespace mcgb {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != MC_OK) throw Error(rc, mc_last_error());
}

class Material {
public:
    Material(const std::string& disp, const std::string& relax, double T) : T_(T) {
        mc_material_h h = nullptr;
        check(mc_material_load(disp.c_str(), relax.c_str(), T, &h));
        h_.reset(h, mc_material_destroy);
        check(mc_material_sums(h_.get(), sums_.data()));
    }
    Material(const std::vector<double>& disp, long nw, long np, const std::vector<double>& relax, double T) : T_(T) {
        mc_material_h h = nullptr;
        check(mc_material_create(disp.data(), nw, np, relax.data(), T, &h));
        h_.reset(h, mc_material_destroy);
        check(mc_material_sums(h_.get(), sums_.data()));
    }
    double temp() const { return T_; }
    double cond() const { return sums_[3]; }
    double energySum() const { return sums_[0]; }
    double fluxSum() const { return sums_[1]; }
    double scatSum() const { return sums_[2]; }
    mc_material_h handle() const { return h_.get(); }

private:
    double T_;
    std::array<double, 4> sums_{};
    std::shared_ptr<mc_material_s> h_;
};

// A domain: subdomains of any shape (Parallelepiped, TriangularPrism,
// Tetrahedron, Prism<N>, Pyramid<N>) plus makePair calls.
class Domain {
public:
    virtual ~Domain() = default;
    long cols() const { return mc_domain_cols(handle()); }
    std::vector<double> cellVolumes() const {
        std::vector<double> v((size_t)cols());
        check(mc_domain_cell_volumes(handle(), v.data()));
        return v;
    }
    mc_domain_h handle() const {
        if (!h_) {
            mc_domain_h h = nullptr;
            check(mc_domain_create_shapes(sdoms_.data(), (int)sdoms_.size(), pairs_.empty() ? nullptr : pairs_.data(),
                                          (int)pairs_.size(), &h));
            h_.reset(h, mc_domain_destroy);
        }
        return h_.get();
    }

protected:
    // a subdomain of any shape: columns are the matrix's columns
    static mc_sdom_desc sdom(int shape, const double o[3], const std::vector<std::array<double, 3>>& cols,
                             const long div[3], const double gradT[3], const std::vector<int>& kind,
                             const std::vector<double>& T) {
        mc_sdom_desc p;
        std::memset(&p, 0, sizeof(p));
        p.shape = shape;
        p.ncols = (int)cols.size();
        for (int i = 0; i < 3; ++i) { p.o[i] = o[i]; p.div[i] = div[i]; p.gradT[i] = gradT[i]; }
        for (size_t c = 0; c < cols.size(); ++c)
            for (int r = 0; r < 3; ++r) p.mat[3 * c + r] = cols[c][r];
        for (size_t f = 0; f < kind.size(); ++f) { p.kind[f] = kind[f]; p.T[f] = f < T.size() ? T[f] : 0.; }
        return p;
    }
    // Parallelepiped with a diagonal matrix (the reference's Diagonal3d)
    static mc_sdom_desc box(const double o[3], const double dim[3], const long div[3], const double gradT[3],
                            const int kind[6], const double T[6]) {
        return sdom(MC_PARALLELEPIPED, o, {{dim[0], 0, 0}, {0, dim[1], 0}, {0, 0, dim[2]}}, div, gradT,
                    std::vector<int>(kind, kind + 6), std::vector<double>(T, T + 6));
    }
    static mc_pair_desc peri(int s1, int f1, int s2, int f2, const double t[3]) {
        mc_pair_desc q;
        std::memset(&q, 0, sizeof(q));
        q.kind = MC_PERI; q.sdom1 = s1; q.face1 = f1; q.sdom2 = s2; q.face2 = f2;
        for (int i = 0; i < 3; ++i) q.transl[i] = t[i];
        q.rot[0] = q.rot[4] = q.rot[8] = 1.;
        return q;
    }
    static mc_pair_desc inter(int s1, int f1, int s2, int f2) {
        mc_pair_desc q;
        std::memset(&q, 0, sizeof(q));
        q.kind = MC_INTER; q.sdom1 = s1; q.face1 = f1; q.sdom2 = s2; q.face2 = f2;
        q.rot[0] = q.rot[4] = q.rot[8] = 1.;
        return q;
    }
    std::vector<mc_sdom_desc> sdoms_;
    std::vector<mc_pair_desc> pairs_;
    mutable std::shared_ptr<mc_domain_s> h_;
};

// FilmDomain: PeriP along x, Diff along y, Spec along z
// (montecarlo/domain.cpp:188-199).
class FilmDomain : public Domain {
public:
    FilmDomain(const double dim[3], const long div[3], double dT) {
        const double o[3] = {0, 0, 0}, g[3] = {-dT / dim[0], 0, 0}, T[6] = {0, 0, 0, 0, 0, 0};
        const int k[6] = {MC_PERI, MC_DIFF, MC_SPEC, MC_PERI, MC_DIFF, MC_SPEC};
        sdoms_.push_back(box(o, dim, div, g, k, T));
        const double t[3] = {dim[0], 0, 0};
        pairs_.push_back(peri(0, 0, 0, 3, t));
    }
};

// BulkDomain: PeriP along x, Spec along y and z (montecarlo/domain.cpp:137-148).
class BulkDomain : public Domain {
public:
    BulkDomain(const double dim[3], const long div[3], double dT) {
        const double o[3] = {0, 0, 0}, g[3] = {-dT / dim[0], 0, 0}, T[6] = {0, 0, 0, 0, 0, 0};
        const int k[6] = {MC_PERI, MC_SPEC, MC_SPEC, MC_PERI, MC_SPEC, MC_SPEC};
        sdoms_.push_back(box(o, dim, div, g, k, T));
        const double t[3] = {dim[0], 0, 0};
        pairs_.push_back(peri(0, 0, 0, 3, t));
    }
};

// HexDomain: Prism<PeriP<Polygon<6>> x 2, Spec x 6> (montecarlo/domain.cpp:238-256).
class HexDomain : public Domain {
public:
    HexDomain(const double dim[4], double dT) {
        const double o[3] = {0, 0, 0}, g[3] = {-dT / dim[0], 0, 0};
        const long div[3] = {0, 0, 0};
        sdoms_.push_back(sdom(MC_PRISM, o,
                              {{dim[0], 0, 0}, {0, dim[1], -dim[3]}, {0, 2 * dim[1], 0}, {0, 2 * dim[1], dim[2]},
                               {0, dim[1], dim[2] + dim[3]}, {0, 0, dim[2]}},
                              div, g, {MC_PERI, MC_PERI, MC_SPEC, MC_SPEC, MC_SPEC, MC_SPEC, MC_SPEC, MC_SPEC}, {}));
        const double t[3] = {dim[0], 0, 0};
        pairs_.push_back(peri(0, 0, 0, 1, t));
    }
};

// PyrDomain: Pyramid<Spec, Spec x 4> (montecarlo/domain.cpp:299-314).
class PyrDomain : public Domain {
public:
    PyrDomain(const double dim[3], double dT) {
        const double o[3] = {0, 0, 0}, g[3] = {-dT / dim[0], 0, 0};
        const long div[3] = {0, 0, 0};
        sdoms_.push_back(sdom(MC_PYRAMID, o,
                              {{dim[0], 0.5 * dim[1], 0.5 * dim[2]}, {0, dim[1], 0}, {0, dim[1], dim[2]}, {0, 0, dim[2]}},
                              div, g, std::vector<int>(5, MC_SPEC), {}));
    }
};

// JctDomain: three blocks, block 0's Rig face paired with two Inter faces
// (montecarlo/domain.cpp:353-383).
class JctDomain : public Domain {
public:
    JctDomain(const double dim[4], const long div[4], double dT) {
        const double g[3] = {-dT / (2 * dim[0]), 0, 0}, T[6] = {0, 0, 0, 0, 0, 0};
        const int k0[6] = {MC_PERI, MC_SPEC, MC_DIFF, MC_PERI, MC_INTER, MC_DIFF};
        const int k1[6] = {MC_PERI, MC_INTER, MC_DIFF, MC_INTER, MC_SPEC, MC_DIFF};
        const int k2[6] = {MC_INTER, MC_INTER, MC_DIFF, MC_PERI, MC_SPEC, MC_DIFF};
        const double o0[3] = {0, 0, 0}, o1[3] = {0, dim[1], 0}, o2[3] = {dim[0], dim[1], 0};
        const double d0[3] = {2 * dim[0], dim[1], dim[3]}, d1[3] = {dim[0], dim[2], dim[3]};
        const long v0[3] = {2 * div[0], div[1], div[3]}, v1[3] = {div[0], div[2], div[3]};
        sdoms_.push_back(box(o0, d0, v0, g, k0, T));
        sdoms_.push_back(box(o1, d1, v1, g, k1, T));
        sdoms_.push_back(box(o2, d1, v1, g, k2, T));
        pairs_.push_back(inter(0, 4, 1, 1));
        pairs_.push_back(inter(0, 4, 2, 1));
        pairs_.push_back(inter(1, 3, 2, 0));
        const double t[3] = {2 * dim[0], 0, 0};
        pairs_.push_back(peri(0, 0, 0, 3, t));
        pairs_.push_back(peri(1, 0, 2, 3, t));
    }
};

// TeeDomain: four blocks (montecarlo/domain.cpp:430-462).
class TeeDomain : public Domain {
public:
    TeeDomain(const double dim[5], const long div[5], double dT) {
        const double g[3] = {-dT / (2 * dim[0] + dim[1]), 0, 0}, T[6] = {0, 0, 0, 0, 0, 0};
        const int k0[6] = {MC_PERI, MC_DIFF, MC_SPEC, MC_INTER, MC_DIFF, MC_SPEC};
        const int k1[6] = {MC_INTER, MC_SPEC, MC_SPEC, MC_INTER, MC_INTER, MC_SPEC};
        const int k2[6] = {MC_DIFF, MC_INTER, MC_SPEC, MC_DIFF, MC_SPEC, MC_SPEC};
        const int k3[6] = {MC_INTER, MC_DIFF, MC_SPEC, MC_PERI, MC_DIFF, MC_SPEC};
        const double o0[3] = {0, 0, 0}, o1[3] = {dim[0], 0, 0}, o2[3] = {dim[0], dim[2], 0},
                     o3[3] = {dim[0] + dim[1], 0, 0};
        const double d0[3] = {dim[0], dim[2], dim[4]}, d1[3] = {dim[1], dim[2], dim[4]}, d2[3] = {dim[1], dim[3], dim[4]};
        const long v0[3] = {div[0], div[2], div[4]}, v1[3] = {div[1], div[2], div[4]}, v2[3] = {div[1], div[3], div[4]};
        sdoms_.push_back(box(o0, d0, v0, g, k0, T));
        sdoms_.push_back(box(o1, d1, v1, g, k1, T));
        sdoms_.push_back(box(o2, d2, v2, g, k2, T));
        sdoms_.push_back(box(o3, d0, v0, g, k3, T));
        pairs_.push_back(inter(0, 3, 1, 0));
        pairs_.push_back(inter(1, 4, 2, 1));
        pairs_.push_back(inter(1, 3, 3, 0));
        const double t[3] = {2 * dim[0] + dim[1], 0, 0};
        pairs_.push_back(peri(0, 0, 3, 3, t));
    }
};

// TubeDomain: three blocks around an open corner, periodic along x
// (montecarlo/domain.cpp:510-540).
class TubeDomain : public Domain {
public:
    TubeDomain(const double dim[4], const long div[4], double dT) {
        const double g[3] = {-dT / dim[0], 0, 0}, T[6] = {0, 0, 0, 0, 0, 0};
        const int k0[6] = {MC_PERI, MC_DIFF, MC_SPEC, MC_PERI, MC_DIFF, MC_INTER};
        const int k1[6] = {MC_PERI, MC_INTER, MC_INTER, MC_PERI, MC_DIFF, MC_DIFF};
        const int k2[6] = {MC_PERI, MC_SPEC, MC_DIFF, MC_PERI, MC_INTER, MC_DIFF};
        const double o0[3] = {0, dim[1], 0}, o1[3] = {0, dim[1], dim[2]}, o2[3] = {0, 0, dim[2]};
        const double d0[3] = {dim[0], dim[3], dim[2]}, d1[3] = {dim[0], dim[3], dim[3]}, d2[3] = {dim[0], dim[1], dim[3]};
        const long v0[3] = {div[0], div[3], div[2]}, v1[3] = {div[0], div[3], div[3]}, v2[3] = {div[0], div[1], div[3]};
        sdoms_.push_back(box(o0, d0, v0, g, k0, T));
        sdoms_.push_back(box(o1, d1, v1, g, k1, T));
        sdoms_.push_back(box(o2, d2, v2, g, k2, T));
        pairs_.push_back(inter(1, 1, 2, 4));
        pairs_.push_back(inter(1, 2, 0, 5));
        const double t[3] = {dim[0], 0, 0};
        pairs_.push_back(peri(0, 0, 0, 3, t));
        pairs_.push_back(peri(1, 0, 1, 3, t));
        pairs_.push_back(peri(2, 0, 2, 3, t));
    }
};

// OctetDomain: one octet-truss cell of 42 subdomains (montecarlo/domain.cpp:
// 591-1238, types montecarlo/domain.h:298-344); dim = (s, d1, d2, t), div =
// (div0 .. div3). average() is OctetDomain::average
// (montecarlo/domain.cpp:1252-1280).
class OctetDomain : public Domain {
public:
    OctetDomain(const double dim[4], const long div[4], double dT) {
        using C = std::array<double, 3>;
        const double r = std::sqrt(2.), h = 0.5, pi = 3.141592653589793;
        const double s = dim[0], t = dim[3];
        const double a = pi / 5. * (dim[1] + dim[2]) - (4. - pi) / 5. * t, b = a / 4.;
        if (!(b > t && a > (r + 1) * (b + t) && s / 2 > a + (r + 1) * (b + t) + t))
            throw Error(MC_ERR_ARG, "Invalid dimensions");
        const double q1 = (r + 1) * h, q2 = (2 + r) * h, ts = t / r;
        const double den = s - 2 * a - 2 * (r + 1) * b - 2 * (2 + r) * t;
        const double g[3] = {dT / den, 0., -dT / den}, z[3] = {0., 0., 0.};
        const long none[3] = {-1, -1, -1};
        const int I = MC_INTER, D = MC_DIFF, S = MC_SPEC, P = MC_PERI;
        const std::vector<std::vector<int>> kinds = {
            {I, P, I, D, S, D}, {D, I, I, D, S, I}, {D, D, I, I, S, S}, {I, P, D, I, I, D}, {I, I, D, I, I, I},
            {I, S, D, D, I, I}, {S, I, P, D, I, D}, {I, D, P, D, I, I}, {D, D, P, I, I, I}, {D, D, I, I, I, I},
            {I, D, I, I, D, I}, {S, I, D, I, D, I}, {D, I, I, S, I}, {I, D, I, S, I}, {I, I, D, S, I},
            {D, D, I, I, S, S}, {D, S, I, D, I, I}, {I, I, I, D, D, I}, {I, D, I, I, D, I}, {D, I, I, I, D, I},
            {D, S, I, D, I, I}, {D, S, I, D, I, I}, {D, I, I, I, D, I}, {I, D, I, I, D, I}, {I, I, I, D, D, I},
            {D, S, I, D, I, I}, {D, D, I, I, S, S}, {I, I, D, S, I}, {I, D, I, S, I}, {D, I, I, S, I},
            {S, I, D, I, D, I}, {I, D, I, I, D, I}, {D, D, I, I, I, I}, {D, D, P, I, I, I}, {I, D, P, D, I, I},
            {S, I, P, D, I, D}, {I, S, D, D, I, I}, {I, I, D, I, I, I}, {I, P, D, I, I, D}, {D, D, I, I, S, S},
            {D, I, I, D, S, I}, {I, P, I, D, S, D}};
        const std::vector<C> e0 = {C{r * t, 0, 0},
                                   C{s / 4 - (2 + r) * h * b - (2 - r) * h * t, s / 4 - (2 + r) * h * (b + t), 0},
                                   C{s / 4 - (2 + r) * h * b - t, s / 4 - (2 + r) * h * b - t, 0}};
        const std::vector<C> e3 = {C{(r + 1) * t, 0, 0}, C{(r + 1) * t, t, 0}, C{t, t, 0}};
        const std::vector<C> e6 = {C{r * t, 0, 0}, C{q1 * b + (r + 1) * t, 0, -q1 * b - t},
                                   C{q1 * b + q2 * t, 0, -q1 * b - q2 * t}};
        const std::vector<C> e10 = {C{(r - 1) * h * b + t / r, 0, -(r - 1) * h * b - t / r},
                                    C{(r - 1) * h * b, 0, -(r - 1) * h * b - r * t}, C{0, 0, -r * t}};
        const C up{-s / 4 + a / 2 + q1 * b + q2 * t, 0, s / 4 - a / 2 - q1 * b - q2 * t};
        const C dn{s / 4 - a / 2 - q1 * b - q2 * t, 0, -s / 4 + a / 2 + q1 * b + q2 * t};
        const std::vector<C> e30 = {C{-(r - 1) * h * b - t / r, 0, (r - 1) * h * b + t / r},
                                    C{-(r - 1) * h * b, 0, (r - 1) * h * b + r * t}, C{0, 0, r * t}};
        const std::vector<C> e34 = {C{-r * t, 0, 0}, C{-q1 * b - (r + 1) * t, 0, q1 * b + t},
                                    C{-q1 * b - q2 * t, 0, q1 * b + q2 * t}};
        const std::vector<C> e37 = {C{-(r + 1) * t, 0, 0}, C{-(r + 1) * t, t, 0}, C{-t, t, 0}};
        const std::vector<C> e40 = {C{-r * t, 0, 0},
                                    C{-s / 4 + (2 + r) * h * b + (2 - r) * h * t, s / 4 - (2 + r) * h * (b + t), 0},
                                    C{-s / 4 + (2 + r) * h * b + t, s / 4 - (2 + r) * h * b - t, 0}};
        auto cat = [](C c0, const std::vector<C>& rest) {
            std::vector<C> v{c0};
            v.insert(v.end(), rest.begin(), rest.end());
            return v;
        };
        int k = 0;
        auto prism = [&](C o, std::vector<C> cols, int shape = MC_PRISM) {
            sdoms_.push_back(sdom(shape, o.data(), cols, none, z, kinds[k], {}));
            ++k;
        };
        auto box = [&](C o, std::vector<C> cols, const long* dv = nullptr) {
            sdoms_.push_back(sdom(MC_PARALLELEPIPED, o.data(), cols, dv ? dv : none, dv ? g : z, kinds[k], {}));
            ++k;
        };
        auto tri = [&](C o, std::vector<C> cols) {
            sdoms_.push_back(sdom(MC_TRIANGULAR_PRISM, o.data(), cols, none, z, kinds[k], {}));
            ++k;
        };
        const long v320[3] = {div[3], div[2], div[0]}, v330[3] = {div[3], div[3], div[0]},
                   v130[3] = {div[1], div[3], div[0]};
        prism({(r + 1) * b + t, b + t, -a}, cat({0, 0, a}, e0));                                        // 00
        prism({(r + 1) * b + t, b + t, -a - t}, cat({0, 0, t}, e0));                                    // 01
        prism({b + t, b + t, -a - t}, {{0, 0, t}, {r * b, 0, 0},
              {s / 4 - (2 - r) * h * b - t, s / 4 - (2 + r) * h * b - t, 0}, {s / 4 - b - t, s / 4 - b - t, 0}});  // 02
        prism({(r + 1) * b, b, -a}, cat({0, 0, a}, e3));                                                // 03
        prism({(r + 1) * b, b, -a - t}, cat({0, 0, t}, e3));                                            // 04
        box({b, b, -a - t}, {{0, 0, t}, {r * b, 0, 0}, {t, t, 0}});                                     // 05
        prism({a, 0, 0}, cat({0, b, 0}, e6));                                                           // 06
        prism({a, b, 0}, cat({0, t, 0}, e6));                                                           // 07
        prism({(r + 1) * (b + t), b, 0}, {{0, t, 0}, {a - (r + 1) * (b + t), 0, 0},
              {a - q1 * b - t / r, 0, -q1 * b - q2 * t}, {0, 0, -a - t}});                              // 08
        prism({b + t, b, -a - t}, {{0, t, 0}, {r * (b + t), 0, 0}, {(r - 1) * h * b + t / r, 0, -q1 * b - t / r},
              {0, 0, -b}});                                                                             // 09
        prism({b + t, b, -a - b - t}, cat({0, t, 0}, e10));                                             // 10
        prism({b + t, 0, -a - b - t}, cat({0, b, 0}, e10));                                             // 11
        tri({b + t, b, -a - b}, {{0, t, 0}, {-t, 0, 0}, {0, 0, b - t}});                                // 12
        prism({b + t, b, -a - b - t}, {{-t, 0, t}, {0, 0, t}, {0, t, t}, {0, t, 0}}, MC_PYRAMID);       // 13
        tri({b + t, b, -a - b - (r + 1) * t}, {{0, t, 0}, {-t, 0, t}, {0, 0, r * t}});                  // 14
        prism({b + t, 0, -a - b - (r + 1) * t}, {{0, 0, r * t}, {0, b, 0}, {-t, b, t}, {-b - t, 0, b + t}});  // 15
        box({s / 4 + a / 2, 0, -s / 4 + a / 2}, {{ts, 0, ts}, {0, b, 0}, up}, v320);                    // 16
        box({s / 4 + a / 2, b, -s / 4 + a / 2}, {{ts, 0, ts}, {0, t, 0}, up}, v330);                    // 17
        box({s / 4 - a / 2, b, -s / 4 - a / 2}, {{a, 0, a}, {0, t, 0}, up}, v130);                      // 18
        box({s / 4 - a / 2 - ts, b, -s / 4 - a / 2 - ts}, {{ts, 0, ts}, {0, t, 0}, up}, v330);          // 19
        box({s / 4 - a / 2 - ts, 0, -s / 4 - a / 2 - ts}, {{ts, 0, ts}, {0, b, 0}, up}, v320);          // 20
        box({s / 4 + a / 2 + ts, 0, -s / 4 + a / 2 + ts}, {{-ts, 0, -ts}, {0, b, 0}, dn}, v320);        // 21
        box({s / 4 + a / 2 + ts, b, -s / 4 + a / 2 + ts}, {{-ts, 0, -ts}, {0, t, 0}, dn}, v330);        // 22
        box({s / 4 + a / 2, b, -s / 4 + a / 2}, {{-a, 0, -a}, {0, t, 0}, dn}, v130);                    // 23
        box({s / 4 - a / 2, b, -s / 4 - a / 2}, {{-ts, 0, -ts}, {0, t, 0}, dn}, v330);                  // 24
        box({s / 4 - a / 2, 0, -s / 4 - a / 2}, {{-ts, 0, -ts}, {0, b, 0}, dn}, v320);                  // 25
        prism({s / 2 - b - t, 0, -s / 2 + a + b + (r + 1) * t}, {{0, 0, -r * t}, {0, b, 0}, {t, b, -t},
              {b + t, 0, -b - t}});                                                                     // 26
        tri({s / 2 - b - t, b, -s / 2 + a + b + (r + 1) * t}, {{0, t, 0}, {t, 0, -t}, {0, 0, -r * t}});  // 27
        prism({s / 2 - b - t, b, -s / 2 + a + b + t}, {{t, 0, -t}, {0, 0, -t}, {0, t, -t}, {0, t, 0}},
              MC_PYRAMID);                                                                              // 28
        tri({s / 2 - b - t, b, -s / 2 + a + b}, {{0, t, 0}, {t, 0, 0}, {0, 0, -b + t}});                // 29
        prism({s / 2 - b - t, 0, -s / 2 + a + b + t}, cat({0, b, 0}, e30));                             // 30
        prism({s / 2 - b - t, b, -s / 2 + a + b + t}, cat({0, t, 0}, e30));                             // 31
        prism({s / 2 - b - t, b, -s / 2 + a + t}, {{0, t, 0}, {-r * (b + t), 0, 0},
              {-(r - 1) * h * b - t / r, 0, q1 * b + t / r}, {0, 0, b}});                               // 32
        prism({s / 2 - (r + 1) * (b + t), b, -s / 2}, {{0, t, 0}, {-a + (r + 1) * (b + t), 0, 0},
              {-a + q1 * b + t / r, 0, q1 * b + q2 * t}, {0, 0, a + t}});                               // 33
        prism({s / 2 - a, b, -s / 2}, cat({0, t, 0}, e34));                                             // 34
        prism({s / 2 - a, 0, -s / 2}, cat({0, b, 0}, e34));                                             // 35
        box({s / 2 - b, b, -s / 2 + a + t}, {{0, 0, -t}, {-r * b, 0, 0}, {-t, t, 0}});                  // 36
        prism({s / 2 - (r + 1) * b, b, -s / 2 + a + t}, cat({0, 0, -t}, e37));                          // 37
        prism({s / 2 - (r + 1) * b, b, -s / 2 + a}, cat({0, 0, -a}, e37));                              // 38
        prism({s / 2 - b - t, b + t, -s / 2 + a + t}, {{0, 0, -t}, {-r * b, 0, 0},
              {-s / 4 + (2 - r) * h * b + t, s / 4 - (2 + r) * h * b - t, 0}, {-s / 4 + b + t, s / 4 - b - t, 0}});  // 39
        prism({s / 2 - (r + 1) * b - t, b + t, -s / 2 + a + t}, cat({0, 0, -t}, e40));                  // 40
        prism({s / 2 - (r + 1) * b - t, b + t, -s / 2 + a}, cat({0, 0, -a}, e40));                      // 41
        const int ip[][4] = {
            {0, 0, 1, 1}, {1, 5, 2, 3}, {0, 2, 3, 4}, {1, 2, 4, 4}, {2, 2, 5, 5}, {3, 0, 4, 1}, {4, 5, 5, 4},
            {3, 3, 8, 5}, {4, 3, 8, 5}, {4, 0, 9, 2}, {5, 0, 9, 2}, {5, 0, 12, 4},
            {6, 1, 7, 0}, {7, 5, 8, 3}, {9, 4, 10, 2}, {10, 0, 11, 1}, {9, 5, 12, 1}, {9, 5, 13, 0}, {10, 5, 14, 1},
            {11, 5, 15, 2}, {12, 2, 13, 2}, {13, 4, 14, 4}, {14, 0, 15, 3},
            {6, 4, 16, 5}, {7, 4, 17, 5}, {8, 4, 18, 5}, {9, 3, 18, 5}, {10, 3, 19, 5}, {11, 3, 20, 5},
            {16, 4, 17, 1}, {17, 0, 18, 3}, {18, 0, 19, 3}, {19, 1, 20, 4},
            {16, 2, 21, 2}, {17, 2, 22, 2}, {18, 2, 23, 2}, {19, 2, 24, 2}, {20, 2, 25, 2},
            {21, 4, 22, 1}, {22, 3, 23, 0}, {23, 3, 24, 0}, {24, 1, 25, 4},
            {21, 5, 30, 3}, {22, 5, 31, 3}, {23, 5, 32, 3}, {23, 5, 33, 4}, {24, 5, 34, 4}, {25, 5, 35, 4},
            {26, 3, 27, 0}, {27, 4, 28, 4}, {28, 2, 29, 2}, {26, 2, 30, 5}, {27, 1, 31, 5}, {28, 0, 32, 5},
            {29, 1, 32, 5}, {30, 1, 31, 0}, {31, 2, 32, 4}, {33, 3, 34, 5}, {34, 0, 35, 1},
            {29, 4, 36, 0}, {32, 2, 36, 0}, {32, 2, 37, 0}, {33, 5, 37, 3}, {33, 5, 38, 3},
            {36, 4, 37, 5}, {37, 1, 38, 0}, {36, 5, 39, 2}, {37, 4, 40, 2}, {38, 4, 41, 2}, {39, 3, 40, 5},
            {40, 1, 41, 0}};
        for (const auto& q : ip) pairs_.push_back(inter(q[0], q[1], q[2], q[3]));
        const int pp[][4] = {{0, 1, 41, 1}, {3, 1, 38, 1}, {6, 2, 35, 2}, {7, 2, 34, 2}, {8, 2, 33, 2}};
        const double tr[3] = {s / 2, 0., -s / 2};
        for (const auto& q : pp) {
            mc_pair_desc x = peri(q[0], q[1], q[2], q[3], tr);
            x.rot[0] = -1.;
            pairs_.push_back(x);
        }
    }
    // OctetDomain::average: the rows averaged over the struts 16-25's
    // first cell layer (third index 0), weighted by cell volume; field is
    // rows x cols column-major.
    std::vector<double> average(const std::vector<double>& field, long rows) const {
        const std::vector<double> cv = cellVolumes();
        std::vector<double> out((size_t)rows, 0.);
        double wsum = 0.;
        long col = 0;
        for (size_t i = 0; i < sdoms_.size(); ++i) {
            const mc_sdom_desc& p = sdoms_[i];
            long n = 0, first = 0;
            if (p.shape == MC_PARALLELEPIPED && p.div[0] >= 0 && p.div[1] >= 0 && p.div[2] >= 0) {
                const long s0 = std::max(p.div[0], 1L), s1 = std::max(p.div[1], 1L), s2 = std::max(p.div[2], 1L);
                n = s0 * s1 * s2;
                first = s0 * s1;
            } else if ((p.shape == MC_PRISM || p.shape == MC_PYRAMID) && p.div[0] >= 0) {
                n = 1;
            } else if ((p.shape == MC_TRIANGULAR_PRISM || p.shape == MC_TETRAHEDRON) && p.div[0] >= 0 &&
                       p.div[1] >= 0 && p.div[2] >= 0) {
                n = std::max(p.div[0], 1L) * std::max(p.div[1], 1L) * std::max(p.div[2], 1L);
            }
            if (i >= 16 && i < 26)
                for (long c = col; c < col + first; ++c) {
                    wsum += cv[(size_t)c];
                    for (long r = 0; r < rows; ++r) out[(size_t)r] += field[(size_t)(c * rows + r)] * cv[(size_t)c];
                }
            col += n;
        }
        for (double& x : out) x /= wsum;
        return out;
    }
};

// Options of the GPU run loop that the reference does not have: the time
// horizon (nsteps x dt), the flight precision, the Philox key and the
// launch shape.
struct RunOptions {
    double dt = 0.5e-12;
    long nsteps = 4000;
    int precision = 32;
    uint64_t seed = 0;
    int stepsPerLaunch = 0;  // 0: the whole horizon in one launch
};

class FieldProblem {
public:
    FieldProblem(const Material& mat, const Domain& dom, long nemit, long maxscat, long maxloop, int kind,
                 long size = 0)
        : mat_(mat), dom_(dom), nemit_(nemit), maxscat_(maxscat), maxloop_(maxloop), kind_(kind), size_(size) {
        if (nemit <= 0 || maxscat <= 0 || maxloop < 0) throw Error(MC_ERR_ARG, "Invalid problem arguments");
        if ((kind == MC_CUMTEMP || kind == MC_CUMFLUX) && (size < 1 || maxscat < 2))
            throw Error(MC_ERR_ARG, "Invalid problem arguments");
    }
    virtual ~FieldProblem() = default;
    long rows() const {
        switch (kind_) {
        case MC_TEMP: return 1;
        case MC_FLUX: return 3;
        case MC_MULTI: return 4;
        case MC_CUMTEMP: return size_ + 1;
        default: return 3 * (size_ + 1);
        }
    }

    // all phonons on the GPU; column-major rows x cols
    std::vector<double> solve(const RunOptions& o = RunOptions(), mc_stats* stats = nullptr) const {
        mc_problem_desc d;
        std::memset(&d, 0, sizeof(d));
        d.problem = kind_;
        d.nemit = nemit_;
        d.maxscat = maxscat_;
        d.maxloop = maxloop_;
        d.dt = o.dt;
        d.nsteps = o.nsteps;
        d.precision = o.precision;
        d.seed = o.seed;
        d.steps_per_launch = o.stepsPerLaunch > 0 ? o.stepsPerLaunch : (int)o.nsteps;
        d.tally_mode = MC_TALLY_AUTO;
        d.cum_size = size_;
        std::vector<double> out((size_t)(rows() * dom_.cols()));
        mc_stats st;
        check(mc_solve(mat_.handle(), dom_.handle(), &d, out.data(), &st));
        if (stats) *stats = st;
        return out;
    }

private:
    const Material& mat_;
    const Domain& dom_;
    long nemit_, maxscat_, maxloop_;
    int kind_;
    long size_;
};

struct TempProblem : FieldProblem {
    TempProblem(const Material& m, const Domain& d, long nemit, long maxscat, long maxloop = 0)
        : FieldProblem(m, d, nemit, maxscat, maxloop, MC_TEMP) {}
};
struct FluxProblem : FieldProblem {
    FluxProblem(const Material& m, const Domain& d, long nemit, long maxscat, long maxloop = 0)
        : FieldProblem(m, d, nemit, maxscat, maxloop, MC_FLUX) {}
};
struct MultiProblem : FieldProblem {
    MultiProblem(const Material& m, const Domain& d, long nemit, long maxscat, long maxloop = 0)
        : FieldProblem(m, d, nemit, maxscat, maxloop, MC_MULTI) {}
};
// montecarlo/problem.h:205-239 (argument order of the reference's constructors)
struct CumTempProblem : FieldProblem {
    CumTempProblem(const Material& m, const Domain& d, long nemit, long size, long maxscat, long maxloop = 0)
        : FieldProblem(m, d, nemit, maxscat, maxloop, MC_CUMTEMP, size) {}
};
struct CumFluxProblem : FieldProblem {
    CumFluxProblem(const Material& m, const Domain& d, long nemit, long size, long maxscat, long maxloop = 0)
        : FieldProblem(m, d, nemit, maxscat, maxloop, MC_CUMFLUX, size) {}
};

}  // namespace mcgb

#endif  // MC_GB300_HPP
