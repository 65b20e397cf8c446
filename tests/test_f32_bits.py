"""Bit-pattern double -> float conversions (csrc/lla_f32_bits.h), checked on the
host with the kernels' own header: sym_to_f32 must round exactly like the
compiler's conversion (round to nearest even) for every double -- random bit
patterns, exact ties between two floats, values either side of each tie, the
edges of the FP32 exponent range (FP32 subnormals, overflow to infinity),
zeros, infinities and NaNs -- and sym_abs_f32 must truncate |a| for the values
sym_f32_range admits."""
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
#include "lla_f32_bits.h"
using namespace lla;
static uint32_t fb(float f) { uint32_t w; std::memcpy(&w, &f, 4); return w; }
static int64_t db(double d) { int64_t b; std::memcpy(&b, &d, 8); return b; }
static long long bad = 0, checked = 0;
static void one(int64_t b) {
    const double d = f64_from_bits(b);
    const float want = (float)d, got = sym_to_f32(b);
    ++checked;
    if (std::isnan(want) ? !std::isnan(got) : fb(want) != fb(got)) {
        if (bad++ < 5) std::printf("mismatch %016llx: %08x vs %08x\n", (unsigned long long)b, fb(want), fb(got));
    }
}
int main() {
    std::mt19937_64 g(12345);
    for (int t = 0; t < 2000000; ++t) one((int64_t)g());  // any bit pattern
    // doubles near FP32 values: the float f, the ties halfway to its neighbours and one ulp either side
    for (int t = 0; t < 1000000; ++t) {
        const uint32_t w = (uint32_t)g();
        float f; std::memcpy(&f, &w, 4);
        if (!std::isfinite(f)) continue;
        const double x = (double)f, up = (double)std::nextafter(f, INFINITY), dn = (double)std::nextafter(f, -INFINITY);
        const double hs[] = {x, 0.5 * (x + up), 0.5 * (x + dn)};
        for (double h : hs) {
            if (!std::isfinite(h)) continue;
            one(db(h));
            one(db(std::nextafter(h, INFINITY)));
            one(db(std::nextafter(h, -INFINITY)));
        }
    }
    // exponent-range edges: FP32 subnormal / normal boundary, FLT_MAX and overflow
    const double edges[] = {0.0, -0.0, 1.1754943508222875e-38, 1.1754942106924411e-38, 1.401298464324817e-45,
                            3.4028234663852886e38, 3.4028235677973366e38, 3.4028236e38, 1e39, -1e39, 1e-46,
                            INFINITY, -INFINITY, NAN};
    for (double e : edges) {
        one(db(e));
        one(db(std::nextafter(e, INFINITY)));
        one(db(std::nextafter(e, -INFINITY)));
    }
    // truncated |a| for the admitted range
    long long tb = 0;
    for (int t = 0; t < 1000000; ++t) {
        const int e = (int)(g() % 201) - 100;
        const double a = std::ldexp(1.0 + (double)(g() >> 12) * 0x1p-52, e);
        const uint64_t v = (uint64_t)db(a);
        if (!sym_f32_range(v)) { std::printf("range\n"); return 1; }
        const float f = sym_abs_f32(v);
        if (!((double)f <= a && (double)std::nextafter(f, INFINITY) > a)) ++tb;
    }
    if (sym_abs_f32(0) != 0.f || sym_f32_range((uint64_t)db(0x1p101)) || sym_f32_range((uint64_t)db(0x1p-101))) {
        std::printf("range edges\n");
        return 1;
    }
    if (bad || tb) { std::printf("bad %lld trunc %lld\n", bad, tb); return 1; }
    std::printf("ok %lld\n", checked);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_bit_conversion_matches_the_compiler():
    d = tempfile.mkdtemp(prefix="lla_f32bits_")
    src, exe = os.path.join(d, "bits.cpp"), os.path.join(d, "bits")
    with open(src, "w") as f:
        f.write(HARNESS)
    # no fast-math: the reference conversions must be IEEE round to nearest even
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC, src, "-o", exe], check=True, timeout=120)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
