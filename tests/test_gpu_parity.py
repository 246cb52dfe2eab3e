"""GPU integrator vs the CPU oracle on the same seeded inputs (all through the C ABI).

Tolerances: the element drift path is compared bit for bit with the oracle
evaluated with the same elementary-function library (precision 2), because
that drift amplifies rounding by ~1e6 in 100 steps; the universal path is
compared at relative 1e-12 per body after 100 steps.
Encounter flags must be identical in both.
"""
import numpy as np
import pytest

import merc
import systems
from oracle import default_params as oparams

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    """Per-body relative difference; bodies that are non-finite in both count
    as equal (the reference's element conversion yields NaN for a few very
    eccentric orbits, src/sim.cuh:90-126 with 8 fixed iterations), a body that
    is non-finite in only one of them counts as a failure."""
    a = a.reshape(3, -1)
    b = b.reshape(3, -1)
    fa, fb = np.isfinite(a).all(0), np.isfinite(b).all(0)
    out = np.zeros(a.shape[1])
    both = fa & fb
    out[both] = np.max(np.abs(a[:, both] - b[:, both]), axis=0) / np.maximum(np.linalg.norm(b[:, both], axis=0),
                                                                             1e-300)
    out[fa != fb] = np.inf
    return out


def run_both(oracle, sysm, steps, **kw):
    kw.setdefault("dt", sysm.dt)
    kw.setdefault("hill_factor", sysm.hill_factor)
    g = merc.Integrator(merc.default_params(**kw))
    g.load_systems(sysm)
    g.step(steps)
    st = g.state()
    gs = g.stats()
    alag = g.a_lag()
    g.close()
    p = oparams(**kw)
    pos, vel, al = oracle.load_elements(p, sysm.body_offset, sysm.n_massive, sysm.mass, sysm.elements, precision=2)
    op, ov, oal, of, ost = oracle.run(p, sysm.body_offset, sysm.n_massive, sysm.mass, pos, vel, al, steps=steps,
                                      precision=2)
    return st, gs, alag, (op, ov, oal, of, ost)


def test_load_matches_oracle(oracle):
    sysm = systems.outer_solar_system()
    g = merc.Integrator(merc.default_params(dt=0.5, hill_factor=3.0))
    g.load_systems(sysm)
    st = g.state()
    p = oparams(dt=0.5, hill_factor=3.0)
    pos, vel, _ = oracle.load_elements(p, sysm.body_offset, sysm.n_massive, sysm.mass, sysm.elements, precision=2)
    assert np.array_equal(st.pos, pos)
    assert np.array_equal(st.vel, vel)


@pytest.mark.parametrize("compat", [0, 7])
def test_elements_outer_system_bitwise(oracle, compat):
    sysm = systems.outer_solar_system()
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_ELEMENTS,
                                                    compat_block=compat)
    assert np.array_equal(st.pos, op), rel_err(st.pos, op).max()
    assert np.array_equal(st.vel, ov)
    assert np.array_equal(alag, oal)
    assert np.array_equal(st.flags, of)


def test_elements_embryo_disk_bitwise(oracle):
    sysm = systems.embryo_disk(n_embryos=254)
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_ELEMENTS)
    assert ost[0] > 0, "the case should exercise close encounters"
    assert gs.ce_body_steps == ost[0]
    assert np.array_equal(st.flags, of)
    assert np.array_equal(st.pos, op), rel_err(st.pos, op).max()
    assert np.array_equal(st.vel, ov)


@pytest.mark.parametrize("rows", [1, 2, 4])
def test_elements_richardson_rows_bitwise(oracle, rows):
    """The exact path's encounter sub-step with 1, 2 and 4 Richardson rows
    (the rows of a big system's encounter body run side by side)."""
    sysm = systems.embryo_disk(n_embryos=254, seed=5)
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 60, drift=merc.DRIFT_ELEMENTS, bs_rows=rows)
    assert ost[0] > 0, "the case should exercise close encounters"
    assert np.array_equal(st.flags, of)
    assert np.array_equal(st.pos, op), rel_err(st.pos, op).max()
    assert np.array_equal(st.vel, ov)


def mixed_batch():
    """One big system (tiled kernels) between small ones (per-body kernels)."""
    a = systems.sweep(n_systems=3, nt_lo=16, nt_hi=40, seed=7)
    b = systems.embryo_disk(n_embryos=94, seed=8)
    c = systems.outer_solar_system(n_test=33, seed=9)
    blocks = []
    for sm in (a, b, c):
        rows = sm.element_rows()
        for s in range(sm.n_systems):
            b0, b1 = sm.body_offset[s], sm.body_offset[s + 1]
            blocks.append((sm.mass[b0:b1], rows[:, b0:b1], int(sm.n_massive[s])))
    out = systems._pack(blocks, 0.02, 3.0, 100, "mixed")
    return out


def two_big_batch():
    """Two big systems (the momentum summed per block, the generic reduce, the
    encounter list over both) and a small one."""
    return systems.concat([systems.embryo_disk(n_embryos=120, seed=41), systems.embryo_disk(n_embryos=70, seed=42),
                           systems.sweep(n_systems=1, nt_lo=10, nt_hi=10, seed=43)])


@pytest.mark.parametrize("which", ["outer", "embryo", "sweep", "mixed", "two_big"])
def test_universal_parity(oracle, which):
    if which == "outer":
        sysm = systems.outer_solar_system()
    elif which == "embryo":
        sysm = systems.embryo_disk(n_embryos=254)
    elif which == "sweep":  # more systems than SMs: the persistent kernel
        sysm = systems.sweep(n_systems=300, nt_lo=4, nt_hi=24)
    elif which == "mixed":
        sysm = mixed_batch()
    else:
        sysm = two_big_batch()
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_UNIVERSAL)
    assert rel_err(st.pos, op).max() <= 1e-12
    assert rel_err(st.vel, ov).max() <= 1e-12
    assert np.array_equal(st.flags, of)
    assert gs.ce_body_steps == ost[0]
    assert gs.kepler_solves == ost[2]
    # the pair sums differ from the oracle's by ulps, which can move a
    # Newton stop by one iteration in rare cases
    assert abs(gs.kepler_iterations - ost[1]) <= max(2, ost[1] // 1000)


@pytest.mark.parametrize("which,steps", [("mixed", 60), ("two_big", 200)])
def test_elements_batches_bitwise(oracle, which, steps):
    """Big and small systems in one batch on the element path: the warp and
    block kernels of the big systems and the per-thread kernels of the small
    ones give the reference's bits (two_big: with close encounters)."""
    sysm = mixed_batch() if which == "mixed" else two_big_batch()
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, steps, drift=merc.DRIFT_ELEMENTS)
    if which == "two_big":
        assert ost[0] > 0, "the case should exercise close encounters"
    assert gs.ce_body_steps == ost[0]
    assert np.array_equal(st.flags, of)
    assert np.array_equal(st.pos, op), rel_err(st.pos, op).max()
    assert np.array_equal(st.vel, ov)
    assert np.array_equal(alag, oal)


@pytest.mark.parametrize("drift,which", [(merc.DRIFT_ELEMENTS, "embryo"), (merc.DRIFT_UNIVERSAL, "embryo"),
                                         (merc.DRIFT_UNIVERSAL, "sweep"), (merc.DRIFT_UNIVERSAL, "two_big")])
def test_split_steps_and_resume_are_exact(drift, which):
    """Steps in one call or several (graph replays of 8 and of 1 step, or
    persistent launches with merged half kicks for small systems) give the
    same bits; so does saving the state and resuming it in a new context."""
    if which == "embryo":
        sysm = systems.embryo_disk(n_embryos=94, seed=12)
    elif which == "two_big":
        sysm = two_big_batch()
    else:  # more systems than SMs: the persistent kernel
        sysm = systems.sweep(n_systems=320, nt_lo=8, nt_hi=60, seed=12)
    kw = dict(dt=sysm.dt, hill_factor=3.0, drift=drift)
    a = merc.Integrator(merc.default_params(**kw))
    a.load_systems(sysm)
    a.step(21)
    sa = a.state()
    b = merc.Integrator(merc.default_params(**kw))
    b.load_systems(sysm)
    b.step(5)
    b.step(3)
    saved = b.state()
    alag = b.a_lag()
    b.close()
    c = merc.Integrator(merc.default_params(**kw))
    c.load_state(sysm.body_offset, sysm.n_massive, sysm.mass, saved.pos, saved.vel, alag)
    c.step(13)
    sc = c.state()
    assert np.array_equal(sa.pos, sc.pos) and np.array_equal(sa.vel, sc.vel)
    a.close()
    c.close()


def test_errors_are_reported_not_crashed():
    g = merc.Integrator(merc.default_params())
    with pytest.raises(merc.MercError) as e:
        g.step(1)
    assert e.value.code == merc.MERC_ERR_STATE
    with pytest.raises(merc.MercError) as e:
        g.load_elements([0, 3], [5], np.ones(3), np.zeros(18))
    assert e.value.code == merc.MERC_ERR_CONFIG
    g.close()


@pytest.mark.parametrize("shape", ["many_small", "few_large", "few_test_particles"])
def test_persistent_sweep_kernel_equals_per_phase_kernels(shape):
    """Small systems run in the persistent kernel (work queue, merged half
    kicks); with the drift log on they run in the per-phase kernels.  Both give
    the same bits: many systems (more than SMs, some cut into two items) and a
    few systems with thousands of test particles (each cut into many items that
    integrate the massive bodies alike, the primary one writing them back)."""
    if shape == "many_small":
        sysm = systems.sweep(n_systems=320, nt_lo=8, nt_hi=120, seed=31)
    elif shape == "few_large":
        sysm = systems.sweep(n_systems=3, nt_lo=3000, nt_hi=6000, seed=32)
    else:  # some systems without test particles
        sysm = systems.sweep(n_systems=200, nt_lo=0, nt_hi=3, seed=33)
    kw = dict(dt=sysm.dt, hill_factor=3.0, drift=merc.DRIFT_UNIVERSAL)
    a = merc.Integrator(merc.default_params(**kw))
    a.load_systems(sysm)
    a.step(30)
    b = merc.Integrator(merc.default_params(**kw))
    b.load_systems(sysm)
    b.mlp_log(1 << 16)  # logging routes small systems through the per-phase kernels
    b.step(30)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa.pos, sb.pos) and np.array_equal(sa.vel, sb.vel)
    assert np.array_equal(sa.flags, sb.flags)
    ta, tb = a.stats(), b.stats()
    assert ta.kepler_iterations == tb.kepler_iterations and ta.ce_body_steps == tb.ce_body_steps
    a.close()
    b.close()


def test_planetesimal_disk_merged_test_particle_kicks(oracle):
    """A big system with many test particles (one source chunk): adjacent half
    kicks of the test particles are merged inside the step graph.  Parity with
    the oracle at 1e-12, and the result does not depend on how the steps are
    split into calls."""
    sysm = systems.planetesimal_disk(seed=41, n_planetesimals=32, n_test=80000)
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 20, drift=merc.DRIFT_UNIVERSAL)
    assert rel_err(st.pos, op).max() <= 1e-12
    assert rel_err(st.vel, ov).max() <= 1e-12
    assert np.array_equal(st.flags, of)
    g = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL))
    g.load_systems(sysm)
    g.step(3)
    g.step(9)
    g.step(8)
    s2 = g.state()
    g.close()
    assert np.array_equal(s2.pos, st.pos, equal_nan=True) and np.array_equal(s2.vel, st.vel, equal_nan=True)


def eccentric_embryo_disk(seed=77, n_embryos=126, n_ecc=40):
    """Embryo disk in which n_ecc embryos move on e = 0.6 orbits: their
    far-field radius follows r_crit near pericentre, so it moves between the
    two kicks around a step boundary."""
    sysm = systems.embryo_disk(seed=seed, n_embryos=n_embryos)
    el = sysm.elements.reshape(6, -1)
    el[4, 2:2 + n_ecc] = 0.6
    return sysm


def test_far_field_recompute_with_eccentric_sources(oracle):
    """Merged kicks reuse the far field of the kick before unless a far-field
    threshold moved; with e = 0.6 sources the second pass runs.  Parity with
    the oracle at 1e-12, and the same bits however the steps are split."""
    sysm = eccentric_embryo_disk()
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_UNIVERSAL)
    assert rel_err(st.pos, op).max() <= 1e-12
    assert rel_err(st.vel, ov).max() <= 1e-12
    assert np.array_equal(st.flags, of)
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    a = merc.Integrator(merc.default_params(**kw))
    a.load_systems(sysm)
    a.step(24)
    assert a.far_recomputes() > 0
    b = merc.Integrator(merc.default_params(**kw))
    b.load_systems(sysm)
    for k in (1, 2, 5, 16):
        b.step(k)
    assert np.array_equal(a.state().pos, b.state().pos) and np.array_equal(a.state().vel, b.state().vel)
    a.close()
    b.close()


def test_programmatic_launches_do_not_change_results():
    """The step graphs with and without programmatic dependent launches give
    the same bits (big system with test particles, and a mixed batch)."""
    for sysm in (systems.planetesimal_disk(seed=43, n_planetesimals=64, n_test=3000), mixed_batch()):
        kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
        out = []
        for on in (True, False):
            g = merc.Integrator(merc.default_params(**kw))
            g.load_systems(sysm)
            g.programmatic_launches(on)
            g.step(19)
            st = g.state()
            out.append((st.pos, st.vel, st.flags))
            g.close()
        assert np.array_equal(out[0][0], out[1][0], equal_nan=True)
        assert np.array_equal(out[0][1], out[1][1], equal_nan=True)
        assert np.array_equal(out[0][2], out[1][2])


def test_encounter_wait_limit_is_reported_and_leaves_the_state_alone():
    """A bounded wait of the encounter task kernel that runs out (its
    predecessor's tasks skipped) is reported, and the integration continues
    with the same bits as without the check."""
    sysm = systems.embryo_disk(seed=11, n_embryos=300)
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    out = []
    for check in (True, False):
        g = merc.Integrator(merc.default_params(**kw))
        g.load_systems(sysm)
        g.step(3)
        if check:
            assert g.encounter_wait_check()
        g.step(9)
        st = g.state()
        out.append((st.pos, st.vel, st.flags, g.stats().ce_body_steps))
        g.close()
    assert out[0][3] > 0
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("steps", [20])
def test_large_small_system_parity(oracle, steps):
    """A batch of small systems whose largest system does not fit in one
    block's shared memory runs the per-phase graphs instead of the persistent
    kernel; parity with the oracle (one 6000-body system among small ones)."""
    a = systems.sweep(n_systems=3, nt_lo=20, nt_hi=40, seed=17)
    b = systems.outer_solar_system(n_test=6000, seed=18)
    sysm = systems.concat([a, b])
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, steps, drift=merc.DRIFT_UNIVERSAL)
    assert rel_err(st.pos, op).max() <= 1e-12
    assert rel_err(st.vel, ov).max() <= 1e-12
    assert np.array_equal(st.flags, of)


@pytest.mark.parametrize("which,eject_r", [("outer", 500.0), ("sweep", 600.0), ("embryo", 1.2)])
@pytest.mark.parametrize("drift", [merc.DRIFT_UNIVERSAL, merc.DRIFT_ELEMENTS])
def test_ejection_and_encounter_flags_match_oracle(oracle, which, eject_r, drift):
    """MERC_FLAG_EJECTED (set when the heliocentric distance is beyond eject_r
    after a step, and kept), MERC_FLAG_CE_LAST / CE_EVER and MERC_FLAG_NONFINITE
    equal the oracle's on the per-body, tiled and persistent paths, and some
    bodies carry each."""
    if which == "outer":
        sysm = systems.outer_solar_system(n_test=200, seed=23)
    elif which == "sweep":
        sysm = systems.sweep(n_systems=12, nt_lo=20, nt_hi=80, seed=24)
    else:
        sysm = systems.embryo_disk(n_embryos=190, seed=25)
    steps = 40
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, steps, drift=drift, eject_r=eject_r)
    assert np.array_equal(st.flags, of)
    ej = (st.flags & merc.FLAG_EJECTED) != 0
    assert 0 < ej.sum() < sysm.n_total
    r = np.linalg.norm(st.pos.reshape(3, -1), axis=0)
    assert np.all(ej[r > eject_r])
    if which == "embryo":
        assert np.any(st.flags & merc.FLAG_CE_EVER)


def test_dense_encounters_match_oracle(oracle):
    """A big system in which about half of the bodies are in an encounter
    every step (changeover at 30 Hill radii): the encounter list built by the
    test kernel from many duplicate flags, and the encounter task kernel with
    ~28 x 60 tasks per step, agree with the oracle."""
    sysm = systems.embryo_disk(n_embryos=120, seed=26)
    steps = 20
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, steps, drift=merc.DRIFT_UNIVERSAL,
                                                    hill_factor=30.0)
    assert gs.ce_body_steps > 0.4 * sysm.n_total * steps
    assert rel_err(st.pos, op).max() <= 1e-12
    assert rel_err(st.vel, ov).max() <= 1e-12
    assert np.array_equal(st.flags, of)


def test_nonfinite_flag_matches_oracle(oracle):
    """A test particle given a NaN eccentricity (no finite state) is flagged
    MERC_FLAG_NONFINITE on both sides, the others are not, and it does not
    disturb them (it is massless)."""
    sysm = systems.outer_solar_system(n_test=30, seed=26)
    el = sysm.elements.reshape(6, -1)
    el[4, 10] = np.nan
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 10, drift=merc.DRIFT_UNIVERSAL)
    assert np.array_equal(st.flags, of)
    nf = (st.flags & merc.FLAG_NONFINITE) != 0
    assert nf[10] and nf.sum() == 1
