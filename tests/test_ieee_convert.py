"""The integer-pipe float <-> double conversions (assist_gb300/csrc/ieee_convert.cuh)
against the compiler's IEEE conversions, bit for bit: random doubles over the
whole exponent range, values a few units from float rounding ties and from the
float range's ends, random floats, zeros, subnormals, infinities and NaN.
The header is plain C++ when compiled without CUDA; g++ compiles the check."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include "ieee_convert.cuh"
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <limits>
static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t nxt() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static uint64_t dbits(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; }
static double dof(uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; }
static uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static float fof(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static long bad = 0, n = 0;
static void chk_d(double x) {
    const float a = ag_d2f_int(x), b = (float)x;
    n++;
    if (fbits(a) != fbits(b) && !(std::isnan(a) && std::isnan(b))) {
        if (bad < 5) std::printf("d2f %a: %a vs %a\n", x, (double)a, (double)b);
        bad++;
    }
}
static void chk_f(float f) {
    const double a = ag_f2d_int(f), b = (double)f;
    n++;
    if (dbits(a) != dbits(b) && !(std::isnan(a) && std::isnan(b))) {
        if (bad < 5) std::printf("f2d %a: %a vs %a\n", (double)f, a, b);
        bad++;
    }
}
int main() {
    for (int i = 0; i < 4000000; i++) chk_d(dof(nxt()));                         // every exponent
    for (int i = 0; i < 4000000; i++) {                                           // float range
        const uint64_t u = nxt();
        const uint64_t e = 1023 - 130 + (u >> 56) % 262;
        chk_d(dof((u & 0x800FFFFFFFFFFFFFull) | (e << 52)));
    }
    for (int i = 0; i < 2000000; i++) {                                           // ties and near ties
        const uint64_t u = nxt();
        const uint64_t e = 1023 - 126 + (u >> 56) % 253;
        const uint64_t m = (u & 0xFFFFFE0000000ull) | 0x10000000ull;              // dropped bits = half
        const uint64_t base = (u & 0x8000000000000000ull) | (e << 52) | m;
        for (int d = -2; d <= 2; d++) chk_d(dof(base + d));
    }
    const double special[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                              3.4028235677973362e38, 1.1754943508222875e-38, 1.1754942e-38, 1.4e-45, 7e-46,
                              1e-300, 1e300, std::numeric_limits<double>::infinity(),
                              -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::quiet_NaN(),
                              std::numeric_limits<double>::denorm_min(), 2.5, 1.0 + 0x1p-24, 1.0 + 0x1p-23 + 0x1p-24};
    for (double x : special) { chk_d(x); chk_d(-x); }
    for (int i = 0; i < 4000000; i++) chk_f(fof((uint32_t)nxt()));
    const float fspecial[] = {0.0f, -0.0f, 1.0f, 1e-45f, 1.17549435e-38f, 3.40282347e38f,
                              std::numeric_limits<float>::infinity(), std::numeric_limits<float>::quiet_NaN()};
    for (float f : fspecial) { chk_f(f); chk_f(-f); }
    std::printf("checked %ld mismatches %ld\n", n, bad);
    return bad != 0;
}
"""


def test_integer_pipe_conversions_match_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "conv.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "conv"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "assist_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout
