"""The Richardson combination's quotients on the GPU: div_known (x / 3,
x / 15, x / 63 by the known-reciprocal correction, merc_device.cuh) equals the
device's IEEE division bit for bit on 4 M inputs per divisor (random
mantissas and exponents, quotients next to powers of two, exact quotients)."""
import numpy as np
import pytest

import merc

pytestmark = pytest.mark.gpu


def _inputs(d, n=4_000_000, seed=5):
    rng = np.random.default_rng(seed)
    mant = rng.uniform(1.0, 2.0, n)
    expo = rng.integers(-1000, 1000, n).astype(np.float64)
    x = mant * np.exp2(expo) * rng.choice([-1.0, 1.0], n)
    near = d * np.exp2(rng.integers(-900, 900, 200_000).astype(np.float64))
    steps = rng.integers(-64, 64, near.size)
    edge = near.copy()
    for k in range(1, 65):  # walk each base value |steps| ulps up or down
        m = np.abs(steps) >= k
        edge[m] = np.nextafter(edge[m], np.where(steps[m] > 0, np.inf, 0.0))
    exact = d * rng.uniform(1.0, 2.0, 100_000) * np.exp2(rng.integers(-900, 900, 100_000).astype(np.float64))
    return np.concatenate([x, edge, -edge, exact, [0.0, -0.0, 2.0 ** -1000, 2.0 ** 1000, 2.0 ** -1001, 5e-324]])


@pytest.mark.parametrize("d,fn", [(3.0, "div3"), (15.0, "div15"), (63.0, "div63")])
def test_known_reciprocal_division_matches_device_division(d, fn):
    x = _inputs(d)
    got = merc.device_math(fn, x)
    ieee = merc.device_math("div", x, np.full_like(x, d))
    host = x / d
    assert np.array_equal(got.view(np.uint64), ieee.view(np.uint64))
    assert np.array_equal(got.view(np.uint64), host.view(np.uint64))
