"""Physical collisions (merc_set_radii; no counterpart in the reference, whose
encounter test only selects the sub-stepper, src/sim.cuh:589-613).

The CPU oracle restates the rule (oracle/merc_oracle.cpp, collide()): after the
drift, bodies in encounter are tested against the massive bodies of their
system, colliding pairs merge in ascending order, the heavier body survives
with the total mass and the mass-weighted position and velocity, the other is
parked.  CPU tests check the rule's conservation laws on the oracle; GPU tests
check the GPU against the oracle at the parity tolerances (element drift bit
for bit, universal drift 1e-12 per body) with identical events, masses and
flags.
"""
import os
import tempfile

import numpy as np
import pytest

import systems
from oracle import default_params as oparams

MERGED, GREW = 16, 32
PARK_R, MERGED_MASS = 1e6, 1e-300


def disk_case():
    """254-body embryo disk with radii inflated to 5e-3 AU (below the 3-Hill
    changeover radius of every pair): three merges in 100 steps."""
    s = systems.embryo_disk(n_embryos=254, seed=5)
    rad = np.full(s.n_total, 5e-3)
    rad[:2] = 5e-4
    return s, rad


def accretion_case():
    """Outer solar system with test particle 0 placed 0.001 rad in mean
    anomaly behind the fourth giant (0.03 AU, deep inside its changeover
    radius) and giant radii of 0.05 AU: accreted in the first step; test
    particle 1 placed 0.1 rad away (3 AU, outside the radius) stays."""
    s = systems.outer_solar_system()
    el = s.element_rows().copy()
    nm = int(s.n_massive[0])
    for tp, dM in ((nm, 1e-3), (nm + 1, 0.1)):
        el[:, tp] = el[:, 3]
        el[3, tp] = el[3, 3] - dM
    s.elements = el.reshape(-1).copy()
    rad = np.zeros(s.n_total)
    rad[:nm] = 0.05
    return s, rad


def oracle_collide(oracle, s, rad, steps, drift, precision=2):
    p = oparams(dt=s.dt, hill_factor=s.hill_factor, drift=drift)
    pos, vel, al = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements, precision=precision)
    return oracle.run_collide(p, s.body_offset, s.n_massive, s.mass, rad, pos, vel, al, steps=steps,
                              precision=precision), (pos, vel, al)


@pytest.mark.parametrize("drift", [0, 1])
def test_oracle_merges_conserve_mass_and_flag(oracle, drift):
    s, rad = disk_case()
    (pos, vel, al, fl, st, mass, ev), _ = oracle_collide(oracle, s, rad, 100, drift)
    assert len(ev) >= 2
    # every event: survivor flagged GREW, absorbed flagged MERGED and parked
    for step, sv, ab in ev:
        assert fl[sv] & GREW and fl[ab] & MERGED
        assert mass[ab] == MERGED_MASS
        # parked on its circular orbit, which it has followed since (~1e-3
        # AU/yr; the element drift's 1e-8 added to h^2, src/sim.cuh:250, tilts
        # it by ~1e-6 rad)
        n = s.n_total
        r = PARK_R + 64 * ab
        assert max(abs(pos[ab] - r), abs(pos[n + ab]), abs(pos[2 * n + ab])) < 1e-5 * r
    assert np.sum(fl & MERGED) // MERGED == len(ev)
    # steps ascending; the total mass is kept (less the parked remainders)
    assert np.all(np.diff(ev[:, 0]) >= 0)
    assert abs(mass.sum() - len(ev) * MERGED_MASS - s.mass.sum()) <= 1e-15 * s.mass.sum()


def test_oracle_zero_radii_change_nothing(oracle):
    s, rad = disk_case()
    p = oparams(dt=s.dt, hill_factor=s.hill_factor, drift=1)
    pos, vel, al = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements, precision=2)
    a = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, al, steps=30, precision=2)
    b = oracle.run_collide(p, s.body_offset, s.n_massive, s.mass, np.zeros(s.n_total), pos, vel, al, steps=30,
                           precision=2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[3], b[3])
    assert len(b[6]) == 0 and np.array_equal(b[5], s.mass)


def test_oracle_merge_keeps_momentum_and_centre_of_mass(oracle):
    """One step from a state where two embryos overlap: the merge step alone
    keeps sum m x and sum m v of the pair (to rounding)."""
    s, _ = disk_case()
    p = oparams(dt=s.dt, hill_factor=s.hill_factor, drift=1)
    pos, vel, al = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements, precision=2)
    n = s.n_total
    a, b = 40, 41
    pos = pos.copy()
    vel = vel.copy()
    for c in range(3):  # body b 1e-4 AU from body a, moving with it
        pos[c * n + b] = pos[c * n + a] + (1e-4 if c == 0 else 0.0)
        vel[c * n + b] = vel[c * n + a]
    rad = np.zeros(n)
    rad[a] = rad[b] = 1e-3
    # no steps of dynamics: compare the merge against the drifted pair by
    # running the same step without radii
    x0, v0, *_ = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, al, steps=1, precision=2)
    out = oracle.run_collide(p, s.body_offset, s.n_massive, s.mass, rad, pos, vel, al, steps=1, precision=2)
    assert out[6].tolist() == [[1, a if s.mass[a] >= s.mass[b] else b, b if s.mass[a] >= s.mass[b] else a]]
    sv = out[6][0][1]
    m = s.mass
    M = m[a] + m[b]
    assert out[5][sv] == M
    # the state after the merge step is the merged drift state advanced by the
    # second jump and kick, which change the pair's momentum by the same
    # (small) amounts either way: check the merged body sits at the centre of
    # mass of the un-merged run to 1e-9 AU
    com = np.array([(m[a] * x0[c * n + a] + m[b] * x0[c * n + b]) / M for c in range(3)])
    got = np.array([out[0][c * n + sv] for c in range(3)])
    assert np.max(np.abs(got - com)) <= 1e-9


@pytest.mark.parametrize("drift", [0, 1])
def test_oracle_test_particle_accretion(oracle, drift):
    s, rad = accretion_case()
    nm = int(s.n_massive[0])
    (pos, vel, al, fl, st, mass, ev), _ = oracle_collide(oracle, s, rad, 5, drift)
    assert ev.tolist() == [[1, 3, nm]]
    assert fl[nm] & MERGED and not fl[nm + 1] & MERGED and fl[3] & GREW
    assert np.array_equal(mass, s.mass)  # a massless body changes no mass


# ---------------------------------------------------------------------------
# GPU against the oracle
# ---------------------------------------------------------------------------
def gpu_collide(s, rad, steps, drift, split=None):
    import merc

    g = merc.Integrator(merc.default_params(dt=s.dt, hill_factor=s.hill_factor, drift=drift))
    g.load_systems(s)
    g.set_radii(rad)
    for k in (split or [steps]):
        g.step(k)
    out = g.state(), g.masses(), g.collisions(), g.a_lag()
    g.close()
    return out


def rel(a, b):
    a = a.reshape(3, -1)
    b = b.reshape(3, -1)
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.linalg.norm(b, axis=0), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("drift", [0, 1])
@pytest.mark.parametrize("case", ["disk", "accretion"])
def test_gpu_collisions_match_oracle(oracle, drift, case):
    s, rad = disk_case() if case == "disk" else accretion_case()
    steps = 100 if case == "disk" else 20
    st, mass, ev, alag = gpu_collide(s, rad, steps, drift)
    (op, ov, oal, of, ost, omass, oev), _ = oracle_collide(oracle, s, rad, steps, drift)
    assert len(oev) >= 1
    assert np.array_equal(ev, oev)
    assert np.array_equal(st.flags, of)
    if drift == 0:
        assert np.array_equal(st.pos, op) and np.array_equal(st.vel, ov) and np.array_equal(mass, omass)
    else:
        assert rel(st.pos, op).max() <= 1e-12 and rel(st.vel, ov).max() <= 1e-12
        assert np.allclose(mass, omass, rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_gpu_collisions_split_calls_and_checkpoint():
    """Collisions give the same bits however the steps are split into calls,
    and a checkpoint taken between them (radii, masses and the event log
    included) resumes to the same bits."""
    import merc

    s, rad = disk_case()
    st_a, m_a, ev_a, _ = gpu_collide(s, rad, 100, merc.DRIFT_UNIVERSAL)
    g = merc.Integrator(merc.default_params(dt=s.dt, hill_factor=s.hill_factor, drift=merc.DRIFT_UNIVERSAL))
    g.load_systems(s)
    g.set_radii(rad)
    g.step(37)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ck.bin")
        g.save_checkpoint(path)
        g.close()
        h = merc.Integrator(merc.default_params())
        h.load_checkpoint(path)
        h.step(63)
        st_b, m_b, ev_b = h.state(), h.masses(), h.collisions()
        h.close()
    assert np.array_equal(st_a.pos, st_b.pos) and np.array_equal(st_a.vel, st_b.vel)
    assert np.array_equal(m_a, m_b) and np.array_equal(ev_a, ev_b)


@pytest.mark.gpu
def test_gpu_radii_off_is_the_plain_step():
    import merc

    s, rad = disk_case()
    a = gpu_collide(s, np.zeros(s.n_total), 30, merc.DRIFT_UNIVERSAL)
    g = merc.Integrator(merc.default_params(dt=s.dt, hill_factor=s.hill_factor, drift=merc.DRIFT_UNIVERSAL))
    g.load_systems(s)
    g.step(30)
    b = g.state()
    g.close()
    assert np.array_equal(a[0].pos, b.pos) and len(a[2]) == 0
