"""The float-pair arithmetic of the FP64 path's stress kernel
(nextsimdg_gb300/csrc/nsdg_pairs.cuh, kMevpStressPairs), against exact
results formed on the host."""
import math

import numpy as np
import pytest

from nextsimdg_gb300.dynamics import selftest_pairs

pytestmark = pytest.mark.gpu


def test_pair_arithmetic_is_near_fp64(gpu):
    rng = np.random.default_rng(11)
    n = 4096
    a = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-8, 5, n)
    x = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-8, 5, n)
    a[::97] = 0.0
    out = selftest_pairs(a, x)
    # representation: |split(a) - a| <= 2^-47 |a|
    assert np.all(np.abs(out[0]) <= 2.0 ** -47 * np.abs(a))
    # widening of a float is exact
    assert np.array_equal(out[1], x.astype(np.float32).astype(np.float64))
    # product: within a few units of 2^-48
    prod = a * x
    assert np.all(np.abs(out[2] - prod) <= 2.0 ** -45 * np.abs(prod) + 1e-300)
    # 9-term dot products with cancellation, against exactly rounded sums
    worst = 0.0
    for i in range(n):
        js = [(i + 7 * k) % n for k in range(9)]
        terms = [a[j] * x[j] for j in js]
        exact = math.fsum(terms)
        mag = sum(abs(t) for t in terms)
        worst = max(worst, abs(out[3][i] - exact) / max(mag, 1e-300))
    assert worst <= 2.0 ** -44, worst
