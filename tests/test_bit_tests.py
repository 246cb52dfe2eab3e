"""The kernels decide several range tests on the bit patterns of doubles
(integer operations) instead of FP64 compares, which take a slot of the FP64
pipe on the GPU: the guarded division's y != 0 and the guarded square root's
x >= 0 (merc_device.cuh), the Stumpff functions' |z| > 0.1 and |z| < 5e-5,
the 0 < x < 1e150 range of r_crit and its thresholds (merc_fast.cuh), the
series guess's window 0.5 p0 < q < 2 p0, and the exact term's K = 1
shortcut.  Each is restated here on numpy's int64 view of the same doubles
and checked against the FP64 compare it replaces, on the edge values (signed
zeros, infinities, NaNs of both signs, subnormals, the largest double, a few
ulps around every threshold) and on random doubles; the shortcut is checked
for the implication it needs (fl(t / b) > 1 and finite)."""
import numpy as np

INF_BITS = 0x7FF0000000000000
SIGN = -0x8000000000000000  # the bits of -0.0 as int64


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def _edges(*thresholds):
    """Special values, and each threshold (both signs) with its four
    neighbouring doubles on either side."""
    out = [0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
           np.finfo(np.float64).max, -np.finfo(np.float64).max, 1.0, -1.0, 0.5, 2.0]
    for c in thresholds:
        for v in (np.float64(c), np.float64(-c)):
            out.append(float(v))
            for direction in (np.inf, -np.inf):
                w = v
                for _ in range(4):
                    with np.errstate(over="ignore"):  # stepping past the largest double
                        w = np.nextafter(w, direction)
                    out.append(float(w))
    return np.array(out, dtype=np.float64)


def _random(n, seed):
    rng = np.random.default_rng(seed)
    raw = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, size=n, dtype=np.int64)
    return raw.view(np.float64)


def test_guarded_division_nonzero():
    x = np.concatenate([_edges(1.0), _random(200000, 1)])
    with np.errstate(invalid="ignore"):
        fp = x != 0.0
    assert np.array_equal((bits(x) << 1) != 0, fp)


def test_guarded_sqrt_nonnegative():
    x = np.concatenate([_edges(1.0), _random(200000, 2)])
    b = bits(x)
    ours = ((b >= 0) & (b <= INF_BITS)) | (b == SIGN)
    with np.errstate(invalid="ignore"):
        fp = x >= 0.0
    assert np.array_equal(ours, fp)


def test_abs_range_tests():
    for c in (0.1, 5e-5):
        x = np.concatenate([_edges(c), _random(200000, 3)])
        a = bits(x) & 0x7FFFFFFFFFFFFFFF
        cb = int(bits(c))
        gt = (a > cb) & (a <= INF_BITS)
        lt = a < cb
        with np.errstate(invalid="ignore"):
            assert np.array_equal(gt, np.abs(x) > c)
            assert np.array_equal(lt, np.abs(x) < c)


def test_positive_below_1e150():
    assert int(bits(1e150)) == 0x5F138D352E5096AF
    x = np.concatenate([_edges(1e150), _random(200000, 4)])
    b = bits(x)
    with np.errstate(invalid="ignore"):
        fp = (x > 0.0) & (x < 1e150)
    assert np.array_equal((b > 0) & (b < 0x5F138D352E5096AF), fp)


def test_series_guess_window():
    rng = np.random.default_rng(5)
    # p0 inside [2^-1020, 2^1022), where the halving and the doubling are
    # exact exponent steps
    p0 = np.concatenate([np.exp2(rng.uniform(-1020, 1022, 4000)), [2.0 ** -1020, np.nextafter(2.0 ** 1022, 0)]])
    for p in p0:
        pb = int(bits(p))
        assert 0x0030000000000000 <= pb < 0x7FD0000000000000
        q = np.concatenate([_edges(0.5 * p, 2.0 * p, p), p * rng.uniform(-3, 3, 50)])
        qb = bits(q)
        ours = (qb > pb - (1 << 52)) & (qb < pb + (1 << 52))
        with np.errstate(invalid="ignore"):
            fp = (q > 0.5 * p) & (q < 2.0 * p)
        assert np.array_equal(ours, fp), p


def test_k_one_shortcut_implies_quotient_above_one():
    rng = np.random.default_rng(6)
    n = 400000
    b = np.exp2(rng.uniform(-1000, 1000, n)) * rng.uniform(1, 2, n)
    # t from 8 ulps below b to 63 above it, then far above it, then random
    near = (bits(b[:20000]) + rng.integers(-8, 64, 20000)).view(np.float64)
    with np.errstate(over="ignore"):
        far = b[20000:] * np.exp2(rng.uniform(-4, 1000, n - 20000))
    t = np.concatenate([near, far, _random(50000, 7)])
    b = np.concatenate([b, b[:50000]])
    tb, bb = bits(t), bits(b)
    with np.errstate(over="ignore"):
        taken = (bb >= 0x0170000000000000) & (bb < INF_BITS) & (tb > bb + 4) & (tb - bb < (996 << 52)) & (tb < INF_BITS)
    assert taken.sum() > 100000
    with np.errstate(over="ignore", invalid="ignore"):
        y = t[taken] / b[taken]
    assert np.all(y > 1.0) and np.all(np.isfinite(y))


def changeover_ranges(y):
    """The changeover weight's three range tests on the bit patterns:
    1 < y < DBL_MAX, -DBL_MAX < y < 0, and 0 <= y <= 1 (changeover_K,
    changeover_K_seeded)."""
    yb = bits(y)
    one, big = int(bits(1.0)), int(bits(np.finfo(np.float64).max))
    above = (yb > one) & (yb < big)
    mag = yb & 0x7FFFFFFFFFFFFFFF
    below = (yb < 0) & (mag != 0) & (mag < big)
    unit = ((yb >= 0) & (yb <= one)) | (yb == SIGN)
    return above, below, unit


def test_changeover_range_tests():
    dmax = np.finfo(np.float64).max
    y = np.concatenate([_edges(1.0, dmax, 0.5), _random(300000, 8)])
    above, below, unit = changeover_ranges(y)
    with np.errstate(invalid="ignore"):
        assert np.array_equal(above, (y > 1.0) & (y < dmax))
        assert np.array_equal(below, (y < 0.0) & (y > -dmax))
        assert np.array_equal(unit, (y >= 0.0) & (y <= 1.0))
