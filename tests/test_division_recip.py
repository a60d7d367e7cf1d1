"""The solve divides by repeated divisors (body masses, the cluster's time
step, per-contact pair counts) through m_div_recip: Markstein's correction
of x * (1 / y) with the divisor's correctly rounded reciprocal.  It must give
the bits of the IEEE division for every operand: random significands
(including the all-ones and power-of-two ones) over a wide exponent range,
integer divisors, the time step, zeros of both signs, subnormals and
infinities.  The harness compiles the library's header for the host (the
same operations, correctly rounded on every IEEE machine)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "delta2_gb300", "csrc")

HARNESS = r"""
#include "d2g_math.cuh"
#include <cstdio>
#include <cstring>
#include <random>
int main() {
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> u(0, 1);
    long bad = 0, n = 0;
    auto chk = [&](double x, double y) {
        const double a = d2g::m_div_recip(x, y, 1.0 / y), b = x / y;
        n++;
        if (d2g::m_bits(a) != d2g::m_bits(b) && !(a != a && b != b)) {
            if (bad < 5) std::printf("mismatch %.17g / %.17g: %.17g vs %.17g\n", x, y, a, b);
            bad++;
        }
    };
    for (int i = 0; i < 2000000; i++) {
        const uint64_t bx = g(), by = g();
        const int ex = (int)(g() % 1201) - 600, ey = (int)(g() % 1201) - 600;
        uint64_t my = by & ((1ull << 52) - 1);
        if (i % 7 == 0) my = (1ull << 52) - 1;
        if (i % 11 == 0) my = 0;
        const uint64_t xb = ((uint64_t)(ex + 1023) << 52) | (bx & ((1ull << 52) - 1)) | (bx >> 63 << 63);
        const uint64_t yb = ((uint64_t)(ey + 1023) << 52) | my;
        double x, y;
        std::memcpy(&x, &xb, 8);
        std::memcpy(&y, &yb, 8);
        chk(x, y);
        chk(x, (double)(1 + g() % 1000));
        chk((u(g) - 0.5) * 1e-3, 0.004166666883975267);
    }
    const double inf = 1.0 / 0.0;
    for (double x : {0.0, -0.0, 1e-310, -1e-310, 4.9e-324, inf, -inf, 1e300, 1.0})
        for (double y : {3.0, 0.004166666883975267, 1e-300, 1e300, 7.0, 1e-310})
            chk(x, y);
    std::printf("cases %ld mismatches %ld\n", n, bad);
    return bad != 0;
}
"""


def test_reciprocal_division_matches_ieee_division(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "div.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "div"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, "-o", str(exe), str(src)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout
