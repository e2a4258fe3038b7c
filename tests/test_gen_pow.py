"""The Zipf sampler's power (gen.h: the series det_log / det_exp / det_pow and
the table-driven tab_log / tab_exp / tab_pow the sampler uses), built from
correctly rounded double +, -, *, / only so that host and GPU draw the same
keys, against the C library's log, exp and pow.  CPU only."""
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
    PowTables tab;
    pow_tables_fill(tab);
    Rng r(12345);
    for (int i = 0; i < 200000; ++i) {
        const double x = std::exp(-700.0 * r.unit()) * (1.0 - 0.5 * r.unit());  // (0, 1]
        const double a = 1.0 + 99.0 * r.unit();                                  // alpha = 1 / (1 - theta)
        const double y = -745.0 * r.unit();
        std::printf("%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", x, a, y, det_log(x),
                    det_exp(y), det_pow(x, a), std::pow(x, a), tab_log(tab, x), tab_exp(tab, y), tab_pow(tab, x, a));
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


@pytest.mark.parametrize("cols", [(3, 4), (7, 8)], ids=["series", "tables"])
def test_log_and_exp_accuracy(samples, cols):
    x, y, lg, ex = samples[:, 0], samples[:, 2], samples[:, cols[0]], samples[:, cols[1]]
    # absolute error a few ulp of max(|ln x|, 1): the power needs the absolute
    # error of a ln x
    assert np.max(np.abs(lg - np.log(x)) / np.maximum(np.abs(np.log(x)), 1.0)) < 6e-16
    ref = np.exp(y)
    normal = ref > 2.3e-308
    assert np.max(np.abs(ex[normal] - ref[normal]) / ref[normal]) < 4e-16 * 745
    assert np.max(np.abs(ex[~normal] - ref[~normal])) <= 5e-324  # subnormal results: within one step


@pytest.mark.parametrize("col", [5, 9], ids=["series", "tables"])
def test_pow_accuracy(samples, col):
    x, a, p, ref = samples[:, 0], samples[:, 1], samples[:, col], samples[:, 6]
    ok = ref > 2.3e-308
    rel = np.abs(p[ok] - ref[ok]) / ref[ok]
    # the exponent a ln x reaches -745: the rounding of ln x and of the product
    # (a few ulp of |a ln x|) bounds the relative error, as for any
    # exp(a log x) evaluation
    bound = (np.abs(a[ok] * np.log(x[ok])) + 4) * 4.5e-16
    assert (rel <= bound).all(), np.max(rel / bound)
    # the sampler's range: results above 1e-9 of the key space
    big = ref[ok] > 1e-9
    assert np.max(rel[big]) < 1e-14
