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

#include <array>
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
