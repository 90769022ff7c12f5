"""CPU test of pbf_gb300/csrc/repeat_add.h: the jump over m sequential
binary32 additions of one value (a float, or an exact product under fma)
gives the bits of the plain loop, for accumulators and addends of either
sign across many binades, shrinking magnitudes and zero crossings, tie
cases (addends with few significant bits), fixed points and non-finite
inputs.  A C++ harness compiled against the header runs both and reports
mismatches."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

HARNESS = r"""
#include <cstdio>
#include <cstdint>
#include <random>
#include "repeat_add.h"
using namespace pbf;
static float naive(float r, float w, uint32_t m) { for (; m; --m) r = ra_add(r, w); return r; }
static float naive_fma(float r, float a, float b, uint32_t m) { for (; m; --m) r = std::fma(a, b, r); return r; }
int main() {
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    long bad = 0, cases = 0;
    auto check = [&](float r, float w, uint32_t m) {
        ++cases;
        const float a = repeat_add(r, w, m), b = naive(r, w, m);
        if (ra_bits(a) != ra_bits(b)) {
            if (bad < 10) std::printf("mismatch r=%a w=%a m=%u: %a vs %a\n", r, w, m, a, b);
            ++bad;
        }
    };
    for (int k = 0; k < 4000; ++k) {
        const float w = (float)std::ldexp(1.0 + u01(g), (int)(u01(g) * 40) - 20);
        const float r = (k % 3 == 0) ? 0.0f : (float)std::ldexp(u01(g), (int)(u01(g) * 50) - 20);
        const uint32_t m = (uint32_t)(u01(g) * ((k % 50 == 0) ? 3000000 : 40000));
        check(r, w, m);
    }
    // addends with few significant bits: ties in some binade
    for (int k = 0; k < 3000; ++k) {
        const int bits = 1 + (int)(u01(g) * 6);
        const double mant = (double)(1 + (uint64_t)(u01(g) * (1 << bits))) / (double)(1 << bits);
        const float w = (float)std::ldexp(mant, (int)(u01(g) * 10) - 5);
        const float r = (float)std::ldexp(u01(g), (int)(u01(g) * 30) - 5);
        check(r, w, (uint32_t)(u01(g) * 200000));
    }
    // either sign, shrinking magnitudes, zero crossings
    for (int k = 0; k < 4000; ++k) {
        const float w = (float)std::ldexp((u01(g) < 0.5 ? -1.0 : 1.0) * (1.0 + u01(g)), (int)(u01(g) * 30) - 15);
        const float r = (float)std::ldexp((u01(g) < 0.5 ? -1.0 : 1.0) * u01(g), (int)(u01(g) * 40) - 10);
        check(r, w, (uint32_t)(u01(g) * 100000));
    }
    // exact products under fma (the delta-p and gradient accumulations)
    long fbad = 0;
    for (int k = 0; k < 3000; ++k) {
        const float a = (float)((u01(g) - 0.5) * std::ldexp(1.0, (int)(u01(g) * 10) - 5));
        const float b = (float)((u01(g) - 0.5) * std::ldexp(1.0, (int)(u01(g) * 10) - 5));
        const float r = (float)((u01(g) - 0.5) * std::ldexp(1.0, (int)(u01(g) * 20) - 5));
        const uint32_t m = (uint32_t)(u01(g) * 100000);
        ++cases;
        const float x = repeat_step(r, m, [a, b](float v) { return std::fma(a, b, v); });
        const float y = naive_fma(r, a, b, m);
        if (ra_bits(x) != ra_bits(y)) {
            if (fbad < 10) std::printf("fma mismatch r=%a a=%a b=%a m=%u: %a vs %a\n", r, a, b, m, x, y);
            ++fbad;
        }
    }
    bad += fbad;
    // the density case: W(0) of h = 1 added up to ~130,000 times from small sums
    const float w0 = 1.5666814f;
    for (uint32_t m : {0u, 1u, 2u, 3u, 7u, 100u, 4095u, 65536u, 130497u, 1000000u})
        for (float r : {0.0f, 1e-3f, 1.0f, 12.5f, 3e5f}) check(r, w0, m);
    // fixed points, zeros and inputs the jump does not take
    check(1e30f, 1.0f, 100000); check(16777216.0f, 1.0f, 1000); check(0.0f, 0.0f, 10);
    check(-5.0f, 0.75f, 20); check(5.0f, -0.75f, 20); check(-0.0f, 1.0f, 5);
    check(1e-40f, 1e-42f, 5000); check(3.0f, 1e-45f, 1000);
    std::printf("%ld cases, %ld mismatches\n", cases, bad);
    return bad != 0;
}
"""


def test_repeat_add_matches_sequential_sum(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "harness.cpp"
    src.write_text(HARNESS.replace("#include <random>", "#include <random>\n#include <cmath>"))
    exe = tmp_path / "harness"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "pbf_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert " 0 mismatches" in out.stdout
