"""The portable sin / cos / acos / log of the oracle (and kernels) stay within
a few ulp of libm over the ranges the hot path uses."""
import math

import numpy as np

from oracle import oracle as O


def ulps(a, b):
    if a == b:
        return 0
    return abs(a - b) / math.ulp(max(abs(a), abs(b), 1e-300))


def test_sin_cos_accuracy():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-4, 4, 3000), rng.uniform(-1e-3, 1e-3, 500), rng.uniform(-200, 200, 500),
                         [0.0, -0.0, math.pi / 4, -math.pi / 4, math.pi / 2, math.pi, 1e-300]])
    worst = 0
    for x in xs:
        worst = max(worst, ulps(O.sin(x), math.sin(x)) if abs(math.sin(x)) > 1e-12 else 0)
        worst = max(worst, ulps(O.cos(x), math.cos(x)) if abs(math.cos(x)) > 1e-12 else 0)
    assert worst <= 4, worst
    assert O.sin(0.0) == 0.0 and O.cos(0.0) == 1.0


def test_acos_accuracy():
    xs = np.concatenate([np.linspace(0, 1, 2001), 1 - np.logspace(-16, -1, 200)])
    for x in xs:
        ref = math.acos(x)
        assert abs(O.acos(x) - ref) <= 8 * math.ulp(max(ref, 1e-3)), x


def test_log_accuracy():
    rng = np.random.default_rng(2)
    for x in np.concatenate([rng.uniform(1e-6, 1, 2000), rng.uniform(1, 1e6, 500)]):
        assert abs(O.log(x) - math.log(x)) <= 4 * math.ulp(abs(math.log(x)) + 1e-300) + 1e-300, x


def test_library_sin_cos_match_oracle_bitwise(tmp_path):
    # The library's portable sin / cos (the header its kernels and host code
    # share, whose sine and cosine series run as one instruction stream) give
    # the oracle's bits for every argument class: reduced and unreduced,
    # every quadrant, tiny, large, non-finite.
    import os
    import shutil
    import subprocess

    if shutil.which("g++") is None:
        import pytest
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "sincos.cpp"
    src.write_text(r'''
#include <cstdio>
#include <cstring>
#include <cstdint>
#include "d2g_math.cuh"
#include "d2o_math.hpp"
static uint64_t bits(double v) { uint64_t b; std::memcpy(&b, &v, 8); return b; }
int main() {
    uint64_t s = 88172645463325252ull, bad = 0, n = 0;
    const double scales[] = {1e-8, 1e-3, 0.7853981633974483, 1.0, 3.2, 10.0, 1e3, 1e8, 2e9};
    for (double sc : scales)
        for (int i = 0; i < 20000; i++) {
            s ^= s << 13; s ^= s >> 7; s ^= s << 17;
            const double x = sc * ((double)(s >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0);
            n += 2;
            bad += bits(d2g::m_sin(x)) != bits(d2o::psin(x));
            bad += bits(d2g::m_cos(x)) != bits(d2o::pcos(x));
        }
    const double special[] = {0.0, -0.0, 1e-300, 0.7853981633974483, 1.5707963267948966, 3.141592653589793,
                              1e9, -1e9, 1.0 / 0.0, -1.0 / 0.0};
    for (double x : special) {
        n += 2;
        const double a = d2g::m_sin(x), b = d2o::psin(x), c = d2g::m_cos(x), d = d2o::pcos(x);
        bad += !(bits(a) == bits(b) || (a != a && b != b));
        bad += !(bits(c) == bits(d) || (c != c && d != d));
    }
    std::printf("%llu %llu\n", (unsigned long long)n, (unsigned long long)bad);
    return 0;
}
''')
    exe = tmp_path / "sincos"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    "-I" + os.path.join(root, "delta2_gb300", "csrc"), "-I" + os.path.join(root, "oracle"),
                    str(src), "-o", str(exe)], check=True)
    n, bad = map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split())
    assert n > 100000 and bad == 0, (n, bad)
