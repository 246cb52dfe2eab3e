"""IEEE binary64 identities behind the exact (reference-order) kernels'
shortcuts, checked on the host's correctly rounded arithmetic (numpy float64
follows the same IEEE rules as the device's add, multiply, divide and square
root):

- stable_div / stable_sqrt (merc_device.cuh) skip the guard's factor 1 and
  addend 0: (netz x) / (y + etz) == (y != 0 ? x / y : (0 x) / (y + 1)) and
  sqrt(x (x >= 0)) == sqrt(x >= 0 ? x : 0 x), bit for bit, NaN, infinities,
  signed zeros and subnormals included;
- exact_term (merc_device.cuh) sets the changeover weight K = 1 without the
  division y = t / b when b >= 2^-1000, t > fl(b (1 + 2^-51)) and
  t < fl(b 1e300): then fl(t / b) is a finite double > 1;
- div_known (merc_device.cuh), the Richardson quotients x / d for d = 3, 15,
  63: q = fl(x y) with y = fl(1 / d), r = x - d q exact, fl(q + r y) equals
  the correctly rounded x / d (Markstein's correction), restated here with
  exact rational arithmetic for the fma steps.
"""
from fractions import Fraction

import numpy as np

SPECIAL = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                    1.7976931348623157e308, -1.7976931348623157e308, 1e-300, 1e300, 0.5, 3.0])


def _bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


def _samples(rng, n):
    # magnitudes over the whole exponent range, both signs, plus special values
    mant = rng.uniform(1.0, 2.0, n)
    expo = rng.integers(-1074, 1024, n).astype(np.float64)
    with np.errstate(over="ignore", under="ignore"):
        x = mant * np.exp2(expo) * rng.choice([-1.0, 1.0], n)
    return np.concatenate([x, SPECIAL])


def test_guarded_division_identity():
    rng = np.random.default_rng(1)
    x = _samples(rng, 200_000)
    y = _samples(rng, 200_000)
    xx, yy = np.meshgrid(SPECIAL, SPECIAL)
    x = np.concatenate([x, xx.ravel()])
    y = np.concatenate([y, yy.ravel()])
    with np.errstate(all="ignore"):
        etz = (y == 0.0).astype(np.float64)
        netz = (y != 0.0).astype(np.float64)
        ref = (netz * x) / (y + etz)
        new = np.where(y != 0.0, x / y, (0.0 * x) / (y + 1.0))
    same = (_bits(ref) == _bits(new)) | (np.isnan(ref) & np.isnan(new))
    assert same.all(), (x[~same][:5], y[~same][:5])


def test_guarded_sqrt_identity():
    rng = np.random.default_rng(2)
    x = _samples(rng, 400_000)
    with np.errstate(all="ignore"):
        ref = np.sqrt(x * (x >= 0.0).astype(np.float64))
        new = np.sqrt(np.where(x >= 0.0, x, x * 0.0))
    same = (_bits(ref) == _bits(new)) | (np.isnan(ref) & np.isnan(new))
    assert same.all(), x[~same][:5]


def test_changeover_division_skip_bound():
    rng = np.random.default_rng(3)
    n = 400_000
    b = np.abs(_samples(rng, n))
    b = b[np.isfinite(b) & (b >= 2.0 ** -1000)]
    # t just above the bound (the critical region) and spread above it
    with np.errstate(all="ignore"):
        lo = b * (1.0 + 2.0 ** -51)
        near = np.nextafter(lo, np.inf)
        spread = lo * rng.uniform(1.0, 4.0, b.size)
        for t in (near, spread, np.nextafter(near, np.inf)):
            ok = (t > b * (1.0 + 2.0 ** -51)) & (t < b * 1e300)
            y = t[ok] / b[ok]
            assert np.isfinite(y).all()
            assert (y > 1.0).all()


def _div_known(x, d, y):
    """div_known with exact fma steps (Fraction arithmetic rounds once)."""
    if not (2.0 ** -1000 <= abs(x) <= 2.0 ** 1000):
        return x / d
    q = x * y  # one rounding, as the device's multiply
    r_exact = Fraction(x) - Fraction(d) * Fraction(q)
    r = float(r_exact)
    assert Fraction(r) == r_exact, "the remainder is not exact"
    if r == 0.0:
        return q
    return float(Fraction(q) + Fraction(r) * Fraction(y))  # fma: one rounding


def test_known_reciprocal_division_is_correctly_rounded():
    rng = np.random.default_rng(4)
    for d in (3.0, 15.0, 63.0):
        y = 1.0 / d
        assert Fraction(y) < Fraction(1) / Fraction(d)  # the reciprocal lies below 1 / d
        mant = rng.uniform(1.0, 2.0, 12_000)
        expo = rng.integers(-990, 990, mant.size).astype(np.float64)
        x = list(mant * np.exp2(expo) * rng.choice([-1.0, 1.0], mant.size))
        # quotients next to powers of two, exact quotients, and the guard's edges
        for k in (-900, -3, 0, 1, 7, 900):
            base = d * 2.0 ** k
            v = base
            for _ in range(40):
                x += [v, -v]
                v = np.nextafter(v, np.inf)
            v = base
            for _ in range(40):
                v = np.nextafter(v, 0.0)
                x += [v]
        x += [0.0, -0.0, 2.0 ** -1000, 2.0 ** 1000, 2.0 ** -1001, 2.0 ** 1001, 5e-324, 1e308]
        for v in x:
            got = _div_known(float(v), d, y)
            want = float(v) / d
            assert np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64), (v, d, got, want)
