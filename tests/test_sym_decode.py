"""The single-system far-field and encounter-test kernels decode their
block-pair task from the block index (sym_decode in merc_kernels.cuh) instead
of loading it from the task list that merc_engine.cu builds: the off-diagonal
pairs I < J row by row, then the diagonal ones.  This restates the decode's
arithmetic (FP32 root estimate, then integer correction steps, FP32 operations
rounded as on the device) and checks it against that order, for every task of
systems up to 80 blocks and of the 63- and 257-block systems of the embryo and
planetesimal disks, and for sampled tasks of larger ones."""
import numpy as np


def _decode(t, nb):
    np_ = nb * (nb - 1) // 2
    if t >= np_:
        return t - np_, t - np_
    f = np.float32
    b = f(2.0) * f(nb) - f(1.0)
    d = f(b * b) - f(8.0) * f(t)
    r = int((b - np.sqrt(max(f(d), f(0.0)))) * f(0.5))
    r = max(0, min(r, nb - 2))
    while r > 0 and r * (2 * nb - r - 1) // 2 > t:
        r -= 1
    while (r + 1) * (2 * nb - r - 2) // 2 <= t:
        r += 1
    return r, t - r * (2 * nb - r - 1) // 2 + r + 1


def _host_order(nb):
    return [(i, j) for i in range(nb) for j in range(i + 1, nb)] + [(i, i) for i in range(nb)]


def test_decode_matches_host_order():
    for nb in list(range(1, 81)) + [63, 257, 600]:
        order = _host_order(nb)
        for t, want in enumerate(order):
            assert _decode(t, nb) == want, (nb, t)


def test_decode_large_systems():
    rng = np.random.default_rng(20261204)
    for nb in (1024, 2047, 2048, 2049, 4096, 5000):
        np_ = nb * (nb - 1) // 2
        ts = np.concatenate([np.arange(0, 64), np.arange(np_ - 64, np_ + nb), rng.integers(0, np_, 4000)])
        for t in ts.tolist():
            i, j = _decode(t, nb)
            if t >= np_:
                assert i == j == t - np_
                continue
            assert 0 <= i < j < nb
            assert i * (2 * nb - i - 1) // 2 + (j - i - 1) == t
