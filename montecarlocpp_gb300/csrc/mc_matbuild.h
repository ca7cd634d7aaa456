// mc_matbuild.h -- the temperature-dependent tables of a Material
// (montecarlo/material.cpp:116-161): relaxation times by the Matthiessen
// sum, dE/dT, the energy, flux and scattering pdfs, their sums, bulk
// conductivity, and the two-level inverse-CDF thresholds the kernels sample
// (montecarlo/material.cpp:51-75). Every formula is a host/device function
// here, evaluated with the same operations in the same order by the host
// build (mc_material_create) and by the device build of many temperatures
// (k_build_materials), so the two give identical bits.
#pragma once

#include <stdint.h>

#include "mc_math.h"

namespace mcg {

// montecarlo/constants.h:18-19
constexpr double MAT_HBAR = 1.054560652927e-034;
constexpr double MAT_KB = 1.380648e-023;
constexpr double MAT_DMIN = 2.2250738585072014e-308;  // smallest normal double
constexpr double MAT_DEPS = 2.220446049250313e-16;    // double epsilon

// 1 / tau of bin (omega, branch p) at T: the two terms c0 w^c1 T^c2
// exp(-c3 / T) of the branch's relaxation row (a term whose c0 is below the
// smallest normal number is left out)
MC_HD inline double tauInverse(const double* relax, long p, double omega, double T) {
    double t = 0.;
    for (int j = 0; j < 2; ++j) {
        const double* c = relax + p * 8 + 4 * j;
        if (c[0] <= MAT_DMIN) continue;
        t += ((c[0] * mcmath::pow(omega, c[1])) * mcmath::pow(T, c[2])) * mcmath::exp(-c[3] / T);
    }
    return t;
}

// dE/dT of one mode: k_B x^2 / (4 sinh^2(x / 2)), x = hbar omega / k_B T
MC_HD inline double dEdT(double omega, double T) {
    const double xs = MAT_HBAR / (MAT_KB * T);
    const double x = xs * omega;
    const double q = x / (2. * mcmath::sinh(x / 2.));
    return MAT_KB * ((x < 0. ? -x : x) < MAT_DEPS ? 1. - x * x / 12. : q * q);
}

// Integer inverse-CDF threshold: T = ceil(cdf * 2^32), so that for a 32-bit
// word x, x < T exactly when x / 2^32 < cdf in FP64.
MC_HD inline unsigned long long cdfThreshold(double cdf) {
    double t = ceil(cdf * 4294967296.0);
    if (t < 0.) t = 0.;
    if (t > 4294967296.0) t = 4294967296.0;
    return (unsigned long long)t;
}

// Branch thresholds of bin w of a pdf (nw x np, row-major): the running sum
// over the branches, each divided by the bin's total. Returns the bin's
// total.
MC_HD inline double branchThresholds(const double* pdf, long w, long np, unsigned long long* pthr) {
    double a = 0.;
    for (long p = 0; p < np; ++p) a += pdf[w * np + p];
    if (!(a > 0.)) {
        for (long p = 0; p < np; ++p) pthr[w * np + p] = 4294967296ull;
        return a;
    }
    double r = 0.;
    for (long p = 0; p < np; ++p) {
        r += pdf[w * np + p];
        pthr[w * np + p] = cdfThreshold(r / a);
    }
    return a;
}

}  // namespace mcg
