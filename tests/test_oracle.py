"""The CPU oracle: pinned to the reference's own source and to closed-form orbits.

- where the reference sources are present, the oracle's binary64 restatement
  (host C library) agrees bit for bit with the reference's src/sim.cuh
  compiled for the host (oracle/_ref), for whole multi-step runs including
  close encounters and the reference's threadIdx quirk;
- everywhere (also without the reference), it agrees with the golden vectors
  that the reference produced (tests/golden/, made by make_golden.py);
- the universal-variable drift (no reference counterpart) matches Kepler's
  equation solved with 40-digit mpmath, and its Stumpff functions match their
  closed forms.
"""
import json
import os

import numpy as np
import pytest

import systems
from oracle import RefHost
from oracle import default_params as oparams

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
needs_ref = pytest.mark.skipif(not RefHost.available(), reason="reference sources not present on this host")


def padded_outer(n_total=112, seed=20261203):
    """Workload 0 padded with far massless bodies to a multiple of 16, the
    shape the reference accepts (N % 16 == 0, mercurius.cu:48)."""
    s = systems.outer_solar_system(seed=seed)
    pad = n_total - s.n_total
    el = s.element_rows()
    padel = np.stack([np.zeros(pad), np.zeros(pad), np.zeros(pad), np.linspace(0, 6, pad), np.full(pad, 0.1),
                      np.linspace(2000, 3000, pad)])
    return np.concatenate([el, padel], axis=1), np.concatenate([s.mass, np.zeros(pad)]), int(s.n_massive[0])


@needs_ref
@pytest.mark.parametrize("block", [112, 7])
def test_oracle_bitwise_vs_reference_outer(oracle, block):
    el, m, nm = padded_outer()
    n = m.size
    R = RefHost()
    rp, rv, ra, rel, ce = R.run(el.reshape(-1), m, nm, block, 0.5, 3.0, 60, want_elements=True)
    p = oparams(dt=0.5, hill_factor=3.0, compat_block=0 if block == n else block)
    off, nmv = np.array([0, n]), np.array([nm])
    pos, vel, alag = oracle.load_elements(p, off, nmv, m, el.reshape(-1))
    op, ov, oa, fl, _ = oracle.run(p, off, nmv, m, pos, vel, alag, steps=60)
    assert np.array_equal(rp, op) and np.array_equal(rv, ov) and np.array_equal(ra, oa)
    assert np.array_equal(rel, oracle.to_elements(p, off, nmv, m, op, ov))
    assert np.array_equal(ce.astype(np.uint32), fl & 1)


@needs_ref
def test_oracle_bitwise_vs_reference_encounters(oracle):
    s = systems.embryo_disk(n_embryos=62, seed=5)
    n, nm = s.n_total, int(s.n_massive[0])
    R = RefHost()
    rp, rv, ra, _, ce = R.run(s.elements, s.mass, nm, n, 0.01, 3.0, 40)
    p = oparams(dt=0.01, hill_factor=3.0)
    pos, vel, alag = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements)
    op, ov, oa, fl, st = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=40)
    assert st[0] > 0, "the case must contain close encounters"
    assert np.array_equal(rp, op) and np.array_equal(rv, ov) and np.array_equal(ra, oa)


@needs_ref
def test_unit_functions_vs_reference(oracle):
    rng = np.random.default_rng(3)
    n = 2000
    M = rng.uniform(0, 2 * np.pi, n)
    e = np.concatenate([rng.uniform(0, 0.99, n - 200), rng.uniform(1.01, 3.0, 200)])
    R = RefHost()
    assert np.array_equal(R.danby(M, e), oracle.danby(M, e, 8))
    el = np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n), M,
                   rng.uniform(0, 0.95, n), rng.uniform(0.3, 1000, n)]).reshape(-1)
    rp, rv = R.cart_from_elem(el)
    op, ov = oracle.cart_from_elem(el, 8)
    assert np.array_equal(rp, op) and np.array_equal(rv, ov)
    assert np.array_equal(R.elem_from_cart(rp, rv), oracle.elem_from_cart(rp, rv))


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_oracle_matches_golden_runs(oracle):
    """Multi-step runs whose expected output was produced by the reference's own
    code (tests/golden/make_golden.py); the oracle must reproduce them bit for bit."""
    g = load_golden("reference_runs.json")
    assert len(g["cases"]) >= 3
    for case in g["cases"]:
        el = np.array(case["elements"])
        m = np.array(case["mass"])
        n, nm = m.size, case["n_massive"]
        p = oparams(dt=case["dt"], hill_factor=case["hill_factor"],
                    compat_block=0 if case["block"] == n else case["block"])
        off, nmv = np.array([0, n]), np.array([nm])
        pos, vel, alag = oracle.load_elements(p, off, nmv, m, el)
        op, ov, oa, fl, _ = oracle.run(p, off, nmv, m, pos, vel, alag, steps=case["steps"])
        assert np.array_equal(op, np.array(case["pos"])), case["name"]
        assert np.array_equal(ov, np.array(case["vel"])), case["name"]
        assert np.array_equal(fl & 1, np.array(case["ce_last"], np.uint32)), case["name"]


def test_oracle_matches_golden_units(oracle):
    g = load_golden("reference_units.json")
    M, e = np.array(g["danby_M"]), np.array(g["danby_e"])
    assert np.array_equal(oracle.danby(M, e, 8), np.array(g["danby_E"]))
    el = np.array(g["elements"])
    op, ov = oracle.cart_from_elem(el, 8)
    assert np.array_equal(op, np.array(g["pos"])) and np.array_equal(ov, np.array(g["vel"]))
    assert np.array_equal(oracle.elem_from_cart(op, ov), np.array(g["elements_back"]))


def kepler_reference(pos, vel, dt):
    """Two-body propagation with mu = 1 by Kepler's equation in 40-digit mpmath."""
    import mpmath as mp

    mp.mp.dps = 40
    r0 = [mp.mpf(float(v)) for v in pos]
    v0 = [mp.mpf(float(v)) for v in vel]
    R = mp.sqrt(sum(x * x for x in r0))
    V2 = sum(x * x for x in v0)
    eta = sum(a * b for a, b in zip(r0, v0))
    alpha = 2 / R - V2  # 1/a
    a = 1 / alpha
    n = mp.sqrt(alpha ** 3)
    # eccentric anomaly at t0 from e cos E = 1 - r/a, e sin E = eta / sqrt(a)
    ecosE = 1 - R / a
    esinE = eta / mp.sqrt(a)
    # Kepler's equation in the difference x = E - E0:
    #   n dt = x - (e cos E0) sin x + (e sin E0) (1 - cos x)
    x = n * dt
    for _ in range(80):
        f = x - ecosE * mp.sin(x) + esinE * (1 - mp.cos(x)) - n * dt
        fp = 1 - ecosE * mp.cos(x) + esinE * mp.sin(x)
        x = x - f / fp
    F = 1 - a / R * (1 - mp.cos(x))
    G = dt + (mp.sin(x) - x) / n
    r1 = [F * p + G * q for p, q in zip(r0, v0)]
    R1 = mp.sqrt(sum(t * t for t in r1))
    Fd = -mp.sqrt(a) / (R * R1) * mp.sin(x)
    Gd = 1 - a / R1 * (1 - mp.cos(x))
    v1 = [Fd * p + Gd * q for p, q in zip(r0, v0)]
    return np.array([float(t) for t in r1]), np.array([float(t) for t in v1])


def test_universal_drift_vs_kepler_equation(oracle):
    rng = np.random.default_rng(11)
    cases = []
    for _ in range(24):
        a = rng.uniform(0.5, 800)
        e = rng.uniform(0, 0.97)
        el = np.array([rng.uniform(0, 1), rng.uniform(0, 6), rng.uniform(0, 6), rng.uniform(0, 6), e, a])
        pos, vel = oracle.cart_from_elem(el, 8)
        period = 2 * np.pi * a ** 1.5
        dt = period * rng.choice([1e-4, 1e-2, 0.3])
        cases.append((pos, vel, dt))
    for pos, vel, dt in cases:
        rp, rv = kepler_reference(pos, vel, dt)
        # converged to machine precision (tol 1e-16): agrees to ~1e-13
        po, vo, its = oracle.universal(pos, vel, dt, tol=1e-16)
        assert np.max(np.abs(po - rp)) <= 1e-13 * np.linalg.norm(rp), (dt, its)
        assert np.max(np.abs(vo - rv)) <= 1e-13 * np.linalg.norm(rv)
        # at the default tolerance (1e-13 on the Newton error estimate of s)
        po, vo, its = oracle.universal(pos, vel, dt)
        assert np.max(np.abs(po - rp)) <= 1e-12 * np.linalg.norm(rp), (dt, its)


def test_stumpff_closed_forms(oracle):
    z = np.concatenate([np.linspace(-30, 30, 121), [1e-12, -1e-12, 0.0]])
    c = oracle.stumpff(z)
    for k, zz in enumerate(z):
        if zz > 1e-8:
            s = np.sqrt(zz)
            ref = [np.cos(s), np.sin(s) / s, (1 - np.cos(s)) / zz, (s - np.sin(s)) / (zz * s)]
        elif zz < -1e-8:
            s = np.sqrt(-zz)
            ref = [np.cosh(s), np.sinh(s) / s, (np.cosh(s) - 1) / -zz, (np.sinh(s) - s) / (-zz * s)]
        else:
            ref = [1.0, 1.0, 0.5, 1.0 / 6.0]
        tol = 1e-9 if abs(zz) < 1e-3 else 1e-12  # the closed forms cancel near 0
        assert np.allclose(c[:, k], ref, rtol=tol, atol=1e-15), zz


def test_long_double_twin_close_to_binary64_universal(oracle):
    s = systems.embryo_disk(n_embryos=62)
    p = oparams(dt=0.01, hill_factor=3.0, drift=1)
    pos, vel, alag = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements)
    a = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=50, precision=0)[0]
    b = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=50, precision=1)[0]
    rel = np.abs(a - b).reshape(3, -1).max(0) / np.linalg.norm(b.reshape(3, -1), axis=0)
    assert rel.max() < 1e-13


def test_product_math_policy_close_to_host_libm(oracle):
    """precision 2 (merc_math functions) and 0 (host libm) run the same algorithm;
    on a well-conditioned (universal) run they agree to rounding."""
    s = systems.outer_solar_system()
    p = oparams(dt=0.5, hill_factor=3.0, drift=1)
    pos, vel, alag = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements)
    pos2, vel2, _ = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements, precision=2)
    assert np.max(np.abs(pos - pos2) / np.maximum(np.abs(pos), 1e-300)) < 1e-14
    a = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=100, precision=0)[0]
    b = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=100, precision=2)[0]
    rel = np.abs(a - b).reshape(3, -1).max(0) / np.linalg.norm(b.reshape(3, -1), axis=0)
    assert rel.max() < 1e-13


def test_stumpff_short_series_for_small_arguments(oracle):
    """Below |z| = 5e-5 the binary64 Stumpff functions use three Taylor terms;
    against the series summed in extended precision they stay within 2 ulp."""
    z = np.concatenate([np.linspace(-5e-5, 5e-5, 201), [4.99e-5, -4.99e-5, 1e-9, -3e-7]])
    c = oracle.stumpff(z)
    zl = z.astype(np.longdouble)
    c2 = np.zeros_like(zl)
    c3 = np.zeros_like(zl)
    f2, f3 = np.longdouble(2), np.longdouble(6)
    term2, term3 = 1 / f2, 1 / f3
    for k in range(8):
        c2 += term2
        c3 += term3
        term2 = -term2 * zl / ((2 * k + 3) * (2 * k + 4))
        term3 = -term3 * zl / ((2 * k + 4) * (2 * k + 5))
    assert np.all(np.abs(c[2] - c2.astype(np.float64)) <= 2 * np.spacing(0.5))
    assert np.all(np.abs(c[3] - c3.astype(np.float64)) <= 2 * np.spacing(1.0 / 6.0))


def test_laguerre_fallback_on_long_drifts(oracle):
    """Drifts long against the pericentre passage (bound orbits of the hard
    drift set with dt = 0.2 yr, x1 = dt / r0^1.5 up to ~14): where 8 Newton
    steps from the plain guess do not converge the solve continues with
    Laguerre-Conway steps, and the result agrees with Kepler's equation in
    40-digit mpmath."""
    s = systems.hard_drifts(n=3 * 2048, seed=8)
    x, v = s.extra["pos"].reshape(3, -1), s.extra["vel"].reshape(3, -1)
    dt = 0.2
    _, _, its = oracle.universal(x.reshape(-1), v.reshape(-1), dt, max_iter=60)
    alpha = 2 / np.linalg.norm(x, axis=0) - (v * v).sum(0)
    long_ones = np.where((its > 8) & (alpha > 0.05))[0]
    assert len(long_ones) >= 10
    for j in long_ones[:12]:
        pos, vel = x[:, j].copy(), v[:, j].copy()
        rp, rv = kepler_reference(pos, vel, dt)
        po, vo, it = oracle.universal(pos, vel, dt, max_iter=60)
        assert it[0] < 60
        assert np.max(np.abs(po - rp)) <= 1e-11 * np.linalg.norm(rp), (j, it)
        assert np.max(np.abs(vo - rv)) <= 1e-11 * np.linalg.norm(rv), (j, it)
