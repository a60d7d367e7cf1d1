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
