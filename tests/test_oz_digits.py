"""Exact-slice digits (csrc/lla_oz_digits.h), checked on the host with the
kernels' own header against an independent restatement: for |a| < 2^e the
magnitude T = floor(|a| 2^(56 - e)) (exact in long double), its eight 7-bit
digits from the top, each signed like a, and the BF16 bits of each signed
digit (the upper half of its FP32 bits; +0 for a zero digit, also when a is
negative).  Random doubles at random distances below their scale, subnormals,
zeros of both signs, values just below the scale, and the packing of four
elements per plane (element 0 in the lowest 16 bits)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "linfa-linalg_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "lla_oz_digits.h"
using namespace lla;
static int64_t db(double d) { int64_t b; std::memcpy(&b, &d, 8); return b; }
static uint16_t bf16_of_int(int d) {  // exact: |d| < 128
    if (d == 0) return 0;
    const float f = (float)d;
    uint32_t w; std::memcpy(&w, &f, 4);
    return (uint16_t)(w >> 16);
}
static long long bad = 0, checked = 0;
static void check4(const double (&a)[4], int e) {
    int64_t b[4];
    for (int u = 0; u < 4; ++u) b[u] = db(a[u]);
    uint32_t q[kOzDigits][2];
    oz_digits_packed4(b, e, q);
    for (int u = 0; u < 4; ++u) {
        const long double T = std::floor(std::ldexp((long double)std::fabs(a[u]), 56 - e));
        unsigned long long t = (unsigned long long)T;
        for (int p = 0; p < kOzDigits; ++p) {
            const int d = (int)((t >> (7 * (kOzDigits - 1 - p))) & 127);
            const uint16_t want = bf16_of_int(std::signbit(a[u]) ? -d : d);
            const uint16_t got = (uint16_t)(q[p][u / 2] >> (16 * (u % 2)));
            ++checked;
            if (want != got && bad++ < 5)
                std::printf("a=%.17g e=%d p=%d: %04x vs %04x\n", a[u], e, p, want, got);
        }
    }
}
int main() {
    std::mt19937_64 g(2024);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (int t = 0; t < 300000; ++t) {
        const int e = (int)(g() % 2001) - 1000;          // the row's scale 2^e
        double a[4];
        for (int u = 0; u < 4; ++u) {
            const int below = (int)(g() % 70);            // |a| in [2^(e-below-1), 2^(e-below))
            double m = 0.5 + 0.5 * U(g);
            if (m >= 1.0) m = 0.5;
            a[u] = std::ldexp(m, e - below) * ((g() & 1) ? -1.0 : 1.0);
        }
        check4(a, e);
    }
    // subnormals under a tiny scale, signed zeros, values just below the scale
    const double tiny[4] = {4.9406564584124654e-324, -2.2250738585072009e-308, 1e-310, -0.0};
    check4(tiny, -1020);
    const double z[4] = {0.0, -0.0, 0.0, -0.0};
    check4(z, 5);
    const double top[4] = {std::nextafter(1.0, 0.0), -std::nextafter(1.0, 0.0), 0.9999, -0.5};
    check4(top, 0);
    if (bad) { std::printf("bad %lld of %lld\n", bad, checked); return 1; }
    std::printf("ok %lld\n", checked);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_packed_digits_match_the_restatement():
    d = tempfile.mkdtemp(prefix="lla_ozdig_")
    src, exe = os.path.join(d, "dig.cpp"), os.path.join(d, "dig")
    with open(src, "w") as f:
        f.write(HARNESS)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC, src, "-o", exe], check=True, timeout=120)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
