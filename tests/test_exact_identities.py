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
  t < fl(b 1e300): then fl(t / b) is a finite double > 1.
"""
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
