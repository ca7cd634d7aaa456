// mc_math.h -- FP64 exp, log, pow and sinh of the Material tables
// (montecarlo/material.cpp:116-161), written with IEEE basic operations
// only (+, -, *, / and exact power-of-two scaling), so that a translation
// unit compiled without contraction (host: -ffp-contract=off; device:
// --fmad=false) gives the same bits on an x86 host, an Arm host and the
// GPU. The host Material build and the device build of many temperatures
// (k_build_materials) both use them, so their tables agree bit for bit.
//
// Methods (published):
// * exp: Cody and Waite's argument reduction x = k ln2 + r with ln 2 split
//   into a short leading part (k ln2_hi exact for |k| < 2^11) and a
//   correction, |r| <= ln2 / 2, then the Taylor series of e^r to r^14
//   (truncation below 2^-60 relative) in Horner form, scaled by 2^k.
// * log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
//   s = (m - 1) / (m + 1), |s| < 0.172, the atanh series to s^25, plus
//   e ln2 (split as above).
// * pow(x, y): binary powering for integer |y| <= 64 (the relaxation-time
//   models' exponents), exp(y log x) otherwise.
// * sinh: its Taylor series below 0.5, (e^h - e^-h) / 2 above.
// Accuracy against the C library: exp within 2 ulp, log and sinh within 3,
// integer powers within 3, the general pow within 64 ulp
// (tests/test_mc_math.py).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MC_HD __host__ __device__
#else
#define MC_HD
#endif

namespace mcg {
namespace mcmath {

MC_HD inline double fromBits(uint64_t b) {
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
}
MC_HD inline uint64_t toBits(double d) {
    uint64_t b;
    memcpy(&b, &d, sizeof b);
    return b;
}

// x * 2^k, exact while the result is a normal number
MC_HD inline double scale2(double x, int k) {
    while (k > 1023) { x *= fromBits((uint64_t)(1023 + 1023) << 52); k -= 1023; }
    while (k < -1022) { x *= fromBits((uint64_t)(1) << 52); k += 1022; }  // 2^-1022
    return x * fromBits((uint64_t)(k + 1023) << 52);
}

// ln 2 = LN2_HI + LN2_LO; LN2_HI has its low 32 bits zero
constexpr double LN2_HI = 6.93147180369123816490e-01;
constexpr double LN2_LO = 1.90821492927058770002e-10;
constexpr double INV_LN2 = 1.44269504088896338700e+00;

MC_HD inline double exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return fromBits(0x7FF0000000000000ull);
    if (x < -745.1332191019412) return 0.0;
    const double kf = floor(x * INV_LN2 + 0.5);
    const int k = (int)kf;
    const double r = (x - kf * LN2_HI) - kf * LN2_LO;
    // Taylor series of e^r, 1/n! for n = 0 .. 14
    double p = 1.0 / 87178291200.0;
    p = p * r + 1.0 / 6227020800.0;
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return scale2(p, k);
}

MC_HD inline double log(double x) {
    if (x != x || x < 0.0) return fromBits(0x7FF8000000000000ull);
    if (x == 0.0) return -fromBits(0x7FF0000000000000ull);
    if (x == fromBits(0x7FF0000000000000ull)) return x;
    int e = 0;
    if (x < fromBits((uint64_t)1 << 52)) {  // subnormal: bring into the normal range
        x *= fromBits((uint64_t)(54 + 1023) << 52);
        e -= 54;
    }
    const uint64_t b = toBits(x);
    e += (int)((b >> 52) & 0x7FF) - 1023;
    double m = fromBits((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);  // [1, 2)
    if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
    const double s = (m - 1.0) / (m + 1.0);
    const double z = s * s;
    // atanh(s) / s = sum z^n / (2n + 1), n = 0 .. 12
    double t = 1.0 / 25.0;
    t = t * z + 1.0 / 23.0;
    t = t * z + 1.0 / 21.0;
    t = t * z + 1.0 / 19.0;
    t = t * z + 1.0 / 17.0;
    t = t * z + 1.0 / 15.0;
    t = t * z + 1.0 / 13.0;
    t = t * z + 1.0 / 11.0;
    t = t * z + 1.0 / 9.0;
    t = t * z + 1.0 / 7.0;
    t = t * z + 1.0 / 5.0;
    t = t * z + 1.0 / 3.0;
    t = t * z + 1.0;
    const double ef = (double)e;
    return (ef * LN2_HI + 2.0 * s * t) + ef * LN2_LO;
}

MC_HD inline double pow(double x, double y) {
    if (y == 0.0) return 1.0;
    const double yi = floor(y);
    if (yi == y && y <= 64.0 && y >= -64.0) {
        int n = (int)(y < 0.0 ? -y : y);
        double r = 1.0, b = x;
        while (n) {
            if (n & 1) r *= b;
            n >>= 1;
            if (n) b *= b;
        }
        return y < 0.0 ? 1.0 / r : r;
    }
    if (x == 0.0) return y > 0.0 ? 0.0 : fromBits(0x7FF0000000000000ull);
    return exp(y * log(x));
}

MC_HD inline double sinh(double h) {
    const double a = h < 0.0 ? -h : h;
    double r;
    if (a < 0.5) {
        // h + h^3 / 3! + ... + h^17 / 17!
        const double z = a * a;
        double t = 1.0 / 355687428096000.0;
        t = t * z + 1.0 / 1307674368000.0;
        t = t * z + 1.0 / 6227020800.0;
        t = t * z + 1.0 / 39916800.0;
        t = t * z + 1.0 / 362880.0;
        t = t * z + 1.0 / 5040.0;
        t = t * z + 1.0 / 120.0;
        t = t * z + 1.0 / 6.0;
        t = t * z + 1.0;
        r = a * t;
    } else {
        const double E = exp(a);
        r = 0.5 * (E - 1.0 / E);
    }
    return h < 0.0 ? -r : r;
}

}  // namespace mcmath
}  // namespace mcg
