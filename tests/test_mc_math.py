"""The FP64 exp, log, pow and sinh of the Material tables
(montecarlocpp_gb300/csrc/mc_math.h), compiled for the host as the library
compiles them (-ffp-contract=off), against the C library on 2e5 random
arguments each: exp within 2 ulp, log and sinh within 3, integer powers
within 3, general powers within 64 ulp (about 1.4e-14 relative)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "montecarlocpp_gb300", "csrc")

PROGRAM = r"""
#include "mc_math.h"
#include <cmath>
#include <cstdio>
#include <random>
using namespace mcg;
static double ulps(double a, double b) {
    if (a == b) return 0;
    return std::fabs(a - b) / (std::fabs(b) * 2.220446049250313e-16);
}
int main() {
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> U(-700, 700), L(-300, 300), S(-20, 20), P(1e9, 1e14), T(10, 1000);
    double me = 0, ml = 0, ms = 0, mp = 0, mg = 0;
    for (int i = 0; i < 200000; ++i) {
        double x = U(g);
        me = std::max(me, ulps(mcmath::exp(x), std::exp(x)));
        double y = std::pow(10.0, L(g));
        ml = std::max(ml, ulps(mcmath::log(y), std::log(y)));
        double h = S(g) * (i % 2 ? 1e-3 : 1);
        ms = std::max(ms, ulps(mcmath::sinh(h), std::sinh(h)));
        double w = P(g);
        mp = std::max(mp, ulps(mcmath::pow(w, (double)(2 + i % 3)), std::pow(w, (double)(2 + i % 3))));
        double t = T(g), e = 0.5 + (i % 9) * 0.37;
        mg = std::max(mg, ulps(mcmath::pow(t, e), std::pow(t, e)));
    }
    std::printf("%.3f %.3f %.3f %.3f %.3f\n", me, ml, ms, mp, mg);
}
"""


def test_mc_math_against_the_c_library(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    me, ml, ms, mp, mg = (float(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                                            check=True).stdout.split())
    assert me <= 2 and ml <= 3 and ms <= 3 and mp <= 3 and mg <= 64, (me, ml, ms, mp, mg)
