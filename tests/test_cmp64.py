"""The integer-pipe double comparisons (hydro_rs_gb300/csrc/cmp64.cuh) give the
truth values of the floating-point comparisons for every pair drawn from
special values (signed zeros, infinities, NaNs, denormals, the extremes) and
random doubles of every sign and magnitude, nearly-equal neighbours included.
The header is plain integer code, compiled here for the host; the device
compiles the same expressions."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "hydro_rs_gb300", "csrc")

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>
#include "cmp64.cuh"

static double from_bits(long long b) { double x; std::memcpy(&x, &b, sizeof x); return x; }

int main() {
    std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0,
                             std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                             std::numeric_limits<double>::quiet_NaN(), -std::numeric_limits<double>::quiet_NaN(),
                             from_bits(0x7ff0000000000001LL), from_bits(0xfff8000000000123LL),
                             std::numeric_limits<double>::denorm_min(), -std::numeric_limits<double>::denorm_min(),
                             std::numeric_limits<double>::min(), -std::numeric_limits<double>::min(),
                             std::numeric_limits<double>::max(), -std::numeric_limits<double>::max(),
                             1e-300, -1e-300, 1e300, -1e300};
    std::mt19937_64 rng(7);
    for (int k = 0; k < 400; k++) {
        double x = from_bits((long long)rng());
        if (std::isnan(x)) continue;
        v.push_back(x);
        v.push_back(std::nextafter(x, 1e308));
        v.push_back(std::nextafter(x, -1e308));
        v.push_back(-x);
    }
    long long bad = 0, n = 0;
    for (double a : v)
        for (double b : v) {
            n++;
            bad += cmp64::lt(a, b) != (a < b);
            bad += cmp64::le(a, b) != (a <= b);
            bad += cmp64::gt(a, b) != (a > b);
            bad += cmp64::ge(a, b) != (a >= b);
            bad += cmp64::eq(a, b) != (a == b);
            bad += cmp64::ne(a, b) != (a != b);
            bad += cmp64::abs_lt(a, b) != (std::fabs(a) < std::fabs(b));
            bad += cmp64::abs_ge(a, b) != (std::fabs(a) >= std::fabs(b));
        }
    std::printf("%lld pairs, %lld mismatches\n", n, bad);
    return bad != 0;
}
"""


def test_cmp64_matches_floating_point_comparisons():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        with open(src, "w") as f:
            f.write(PROGRAM)
        subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
