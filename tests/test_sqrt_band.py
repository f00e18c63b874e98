"""sc_sqrt_le_test (scmath.h): the neighbour scans decide sqrtf(x) <= d from
x against two bounds around d*d and take sqrtf only between them.  The
answer must equal sqrtf(x) <= d for every x; this compiles the header for the
host and checks x stepped float by float around both bounds and around d*d,
plus random and special values, for a spread of d."""
import os
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "spatial_cell_gb300", "csrc")

PROGRAM = r"""
#include "scmath.h"
#include <cstdio>
#include <cmath>
#include <cstdint>
#include <limits>

static long bad = 0, checked = 0;
static void check(float d, float x) {
    const sc_sqrt_le s = sc_sqrt_le_make(d);
    const bool got = sc_sqrt_le_test(s, x), want = sqrtf(x) <= d;
    checked++;
    if (got != want && bad++ < 10) std::printf("mismatch d=%a x=%a got=%d want=%d\n", d, x, got, want);
}
static void around(float d, float c) {
    float lo = c, hi = c;
    for (int k = 0; k < 96; k++) {
        check(d, lo);
        check(d, hi);
        lo = std::nextafterf(lo, 0.0f);
        hi = std::nextafterf(hi, INFINITY);
    }
}
int main() {
    uint64_t st = 0x9e3779b97f4a7c15ull;
    auto rnd = [&]() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; };
    const float fixed[] = {1.0f, 2.0f, 3.0f, 5.5f, 6.0f, 0.7f, 1.9f, 3.4199998f, 1e-10f, 1e10f,
                           9.999999e-11f, 1.0000001e10f, 1e-20f, 1e20f, 0.0f, -0.0f, -1.0f,
                           std::numeric_limits<float>::denorm_min(), INFINITY, -INFINITY, NAN};
    float ds[4096];
    int nd = 0;
    for (float d : fixed) ds[nd++] = d;
    while (nd < 4096) {
        // random d over [2^-40, 2^40]: exponent and mantissa drawn separately
        const uint32_t e = 87u + (uint32_t)(rnd() % 81u), m = (uint32_t)(rnd() & 0x7fffffu);
        const uint32_t u = (e << 23) | m;
        float d;
        std::memcpy(&d, &u, 4);
        ds[nd++] = d;
    }
    for (int k = 0; k < nd; k++) {
        const float d = ds[k];
        const sc_sqrt_le s = sc_sqrt_le_make(d);
        around(d, d * d);
        if (std::isfinite(s.lo)) around(d, s.lo);
        if (std::isfinite(s.hi)) around(d, s.hi);
        const float sp[] = {0.0f, -0.0f, INFINITY, NAN, std::numeric_limits<float>::denorm_min(),
                            std::numeric_limits<float>::max()};
        for (float x : sp) check(d, x);
        for (int r = 0; r < 64; r++) {
            const float x = (float)(rnd() % 1000000u) * 1e-6f * 4.0f * (std::isfinite(d) ? d * d : 1.0f);
            check(d, x);
        }
    }
    std::printf("checked %ld bad %ld\n", checked, bad);
    return bad != 0;
}
"""


def test_sqrt_band_equals_sqrtf_comparison():
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "band.cpp")
        exe = os.path.join(tmp, "band")
        with open(src, "w") as f:
            f.write(PROGRAM.replace("#include <cstdint>", "#include <cstdint>\n#include <cstring>"))
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC, src, "-o", exe],
                           capture_output=True, text=True)
        if r.returncode != 0:
            pytest.fail("compile failed:\n" + r.stderr)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "bad 0" in r.stdout
