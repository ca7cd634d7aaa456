// mc_main.cpp -- command line driver with the reference's argument grammar
// for the field problems (montecarlo/main.cpp:216-235,254-472), running
// every phonon through the GB300 kernels via the C++ mirror in
// include/mc_gb300.hpp.
//
//   mc_main prefix silicon|grey T               (Si_* / grey_* files)
//           | custom T disp relax
//           film dim0 dim1 div1 | bulk dim0 div0
//           temp|flux|multi nemit maxscat maxloop nsim
//           | cumtemp|cumflux nemit size maxscat maxloop nsim
//           [dt nsteps precision seed]
//
// The trailing four arguments are the GPU run loop's time horizon
// (nsteps x dt), flight precision and Philox key; nsim > 1 prints the mean
// and standard deviation of nsim solves (montecarlo/main.cpp:181-210).
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mc_gb300.hpp"

namespace {

void printSolution(const std::vector<double>& sol, long rows, long cols) {
    // montecarlo/main.cpp:67-84: rows of %16.9e
    for (long i = 0; i < rows; ++i) {
        for (long j = 0; j < cols; ++j) std::printf("%16.9e ", sol[(size_t)(j * rows + i)]);
        std::printf("\n");
    }
    std::printf("\n");
}

int usage() {
    std::fprintf(stderr,
                 "usage: mc_main prefix silicon|grey T | custom T disp relax  film dim0 dim1 div1 | bulk dim0 div0"
                 "  temp|flux|multi nemit maxscat maxloop nsim | cumtemp|cumflux nemit size maxscat maxloop nsim"
                 "  [dt nsteps precision seed]\n");
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2 || std::string(argv[1]) == "--help") return usage();
    std::stringstream ss;
    for (int i = 1; i < argc; ++i) ss << argv[i] << ' ';
    std::string prefix, matStr, domStr, probStr;
    double T = 300.;
    ss >> prefix >> matStr >> T;
    if (chdir(prefix.c_str()) != 0) {
        std::fprintf(stderr, "Invalid directory\n");
        return 1;
    }
    try {
        std::string disp, relax;
        if (matStr == "silicon") { disp = "Si_disp.txt"; relax = "Si_relax2.txt"; }
        else if (matStr == "grey") { disp = "grey_disp.txt"; relax = "grey_relax2.txt"; }
        else if (matStr == "custom") ss >> disp >> relax;
        else { std::fprintf(stderr, "Invalid material\n"); return 1; }
        mcgb::Material mat(disp, relax, T);
        ss >> domStr;
        std::unique_ptr<mcgb::Domain> dom;
        if (domStr == "film") {
            double dim[3]; long div[3] = {0, 0, 0};
            ss >> dim[0] >> dim[1] >> div[1];
            dim[2] = dim[0];
            dom.reset(new mcgb::FilmDomain(dim, div, 1e6 * dim[0]));
        } else if (domStr == "bulk") {
            double d0; long div[3] = {0, 0, 0};
            ss >> d0 >> div[0];
            double dim[3] = {d0, d0, d0};
            dom.reset(new mcgb::BulkDomain(dim, div, 1e6 * d0));
        } else if (domStr == "hex") {  // montecarlo/main.cpp:320-328
            double dim[4];
            ss >> dim[0] >> dim[1];
            dim[2] = dim[3] = dim[1];
            dom.reset(new mcgb::HexDomain(dim, 1e6 * dim[0]));
        } else if (domStr == "pyr") {  // montecarlo/main.cpp:330-337
            double dim[3];
            ss >> dim[0] >> dim[1];
            dim[2] = dim[1];
            dom.reset(new mcgb::PyrDomain(dim, 1e6 * dim[0]));
        } else if (domStr == "jct") {  // montecarlo/main.cpp:339-348
            double dim[4];
            long div[4] = {0, 0, 0, 0};
            ss >> dim[0] >> dim[3];
            dim[1] = dim[2] = dim[0];
            dom.reset(new mcgb::JctDomain(dim, div, 2e6 * dim[0]));
        } else if (domStr == "tee") {  // montecarlo/main.cpp:350-362
            double d0;
            double dim[5];
            long div0;
            ss >> d0 >> dim[4] >> div0;
            dim[0] = dim[1] = dim[2] = dim[3] = d0;
            long div[5] = {div0, div0, div0, div0, 0};
            dom.reset(new mcgb::TeeDomain(dim, div, 3e6 * d0));
        } else if (domStr == "tube") {  // montecarlo/main.cpp:364-374
            double dim[4];
            long div[4] = {0, 0, 0, 0};
            ss >> dim[0] >> dim[1] >> dim[3] >> div[1] >> div[3];
            dim[2] = dim[1];
            div[2] = div[1];
            dom.reset(new mcgb::TubeDomain(dim, div, 1e6 * dim[0]));
        } else if (domStr == "octet") {  // montecarlo/main.cpp:376-386
            double dim[4];
            long div[4];
            double dT;
            ss >> dim[0] >> dim[1] >> dim[2] >> dim[3] >> div[0] >> div[1] >> div[2] >> div[3] >> dT;
            if (!(dim[0] > 0 && dim[1] > 0 && dim[2] > 0 && dim[3] > 0)) {
                std::fprintf(stderr, "Dimensions must be positive\n");
                return 1;
            }
            dom.reset(new mcgb::OctetDomain(dim, div, dT));
        } else {
            std::fprintf(stderr, "Invalid domain (this driver serves film, bulk, hex, pyr, jct, tee, tube and octet)\n");
            return 1;
        }
        long nemit = 0, maxscat = 0, maxloop = 0, nsim = 1, size = 0;
        ss >> probStr >> nemit;
        if (probStr == "cumtemp" || probStr == "cumflux") ss >> size;  // montecarlo/main.cpp:446-456
        ss >> maxscat >> maxloop >> nsim;
        if (!ss) { std::fprintf(stderr, "Invalid problem arguments\n"); return 1; }
        mcgb::RunOptions o;
        double dt;
        long nsteps;
        int prec;
        unsigned long long seed;
        if (ss >> dt >> nsteps >> prec >> seed) { o.dt = dt; o.nsteps = nsteps; o.precision = prec; o.seed = seed; }
        std::unique_ptr<mcgb::FieldProblem> prob;
        if (probStr == "temp") prob.reset(new mcgb::TempProblem(mat, *dom, nemit, maxscat, maxloop));
        else if (probStr == "flux") prob.reset(new mcgb::FluxProblem(mat, *dom, nemit, maxscat, maxloop));
        else if (probStr == "multi") prob.reset(new mcgb::MultiProblem(mat, *dom, nemit, maxscat, maxloop));
        else if (probStr == "cumtemp") prob.reset(new mcgb::CumTempProblem(mat, *dom, nemit, size, maxscat, maxloop));
        else if (probStr == "cumflux") prob.reset(new mcgb::CumFluxProblem(mat, *dom, nemit, size, maxscat, maxloop));
        else { std::fprintf(stderr, "Invalid problem\n"); return 1; }
        const long rows = prob->rows(), cols = dom->cols();
        std::vector<double> mean((size_t)(rows * cols), 0.), m2((size_t)(rows * cols), 0.);
        for (long n = 0; n < std::max(1L, nsim); ++n) {
            mcgb::RunOptions on = o;
            on.seed = o.seed + (unsigned long long)n;
            mc_stats st;
            std::vector<double> sol = prob->solve(on, &st);
            std::printf("Solution %ld (%ld phonons, %.6g phonon-steps, %.3f ms)\n", n, st.nemit, st.phonon_steps,
                        st.kernel_ms);
            printSolution(sol, rows, cols);
            // Welford (montecarlo/field.cpp:255-262)
            for (size_t i = 0; i < sol.size(); ++i) {
                double d = sol[i] - mean[i];
                mean[i] += d / (double)(n + 1);
                m2[i] += d * (sol[i] - mean[i]);
            }
        }
        if (nsim > 1) {
            std::printf("Mean\n");
            printSolution(mean, rows, cols);
            for (double& x : m2) x = std::sqrt(x / (double)(nsim - 1));
            std::printf("Standard Deviation\n");
            printSolution(m2, rows, cols);
        }
    } catch (const mcgb::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
