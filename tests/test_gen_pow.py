"""The Zipf sampler's power (gen.h): the series det_log / det_exp / det_pow
(double +, -, *, / only; they fill the tables) and the fixed-point
fix_pow_floor the sampler uses (integer only), so that host and GPU draw the
same keys, against the C library's log, exp and pow.  CPU only."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHECK = r"""
#include <cmath>
#include <cstdio>
#include "gen.h"
using namespace ltpg::gen;
int main() {
    FixTables tab;
    fix_tables_fill(tab);
    Rng r(12345);
    for (int i = 0; i < 200000; ++i) {
        // (0, 1]: half over the whole range, half near 1 (the sampler's range)
        const double x = (i & 1) ? std::exp(-700.0 * r.unit()) * (1.0 - 0.5 * r.unit()) : std::exp(-0.3 * r.unit());
        const double a = 1.0 + 99.0 * r.unit();                                  // alpha = 1 / (1 - theta)
        const double y = -745.0 * r.unit();
        const unsigned long long n = 1ull << 40;
        std::printf("%.17g %.17g %.17g %.17g %.17g %.17g %.17g %llu %.21Lg\n", x, a, y, det_log(x), det_exp(y),
                    det_pow(x, a), std::pow(x, a), (unsigned long long)fix_pow_floor(tab, x, a, n),
                    (long double)n * std::pow((long double)x, (long double)a));
    }
}
"""


@pytest.fixture(scope="module")
def samples(tmp_path_factory):
    d = tmp_path_factory.mktemp("pow")
    src, exe = d / "check.cpp", d / "check"
    src.write_text(CHECK)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "ltpg_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return np.array([list(map(float, ln.split())) for ln in out.splitlines()])


def test_log_and_exp_accuracy(samples):
    x, y, lg, ex = samples[:, 0], samples[:, 2], samples[:, 3], samples[:, 4]
    # absolute error a few ulp of max(|ln x|, 1): the power needs the absolute
    # error of a ln x
    assert np.max(np.abs(lg - np.log(x)) / np.maximum(np.abs(np.log(x)), 1.0)) < 6e-16
    ref = np.exp(y)
    normal = ref > 2.3e-308
    assert np.max(np.abs(ex[normal] - ref[normal]) / ref[normal]) < 4e-16 * 745
    assert np.max(np.abs(ex[~normal] - ref[~normal])) <= 5e-324  # subnormal results: within one step


def test_pow_accuracy(samples):
    x, a, p, ref = samples[:, 0], samples[:, 1], samples[:, 5], samples[:, 6]
    ok = ref > 2.3e-308
    rel = np.abs(p[ok] - ref[ok]) / ref[ok]
    # the exponent a ln x reaches -745: the rounding of ln x and of the product
    # (a few ulp of |a ln x|) bounds the relative error, as for any
    # exp(a log x) evaluation
    bound = (np.abs(a[ok] * np.log(x[ok])) + 4) * 4.5e-16
    assert (rel <= bound).all(), np.max(rel / bound)


def test_fixed_point_power(samples):
    """floor(2^40 x^a) in fixed point against long-double pow: off by at most
    a couple of units or a few parts in 1e15, and exactly 0 where x^a < 2^-40."""
    x, a = samples[:, 0], samples[:, 1]
    fix = samples[:, 7]
    ref = samples[:, 8]
    big = ref >= 1.0
    err = np.abs(fix[big] - np.floor(ref[big]))
    assert (err <= np.maximum(2.0, ref[big] * 3e-15 * (1 + np.abs(a[big] * np.log(x[big])) / 8))).all()
    assert (fix[ref < 1.0] == 0).all()
    assert big.sum() > 1000
