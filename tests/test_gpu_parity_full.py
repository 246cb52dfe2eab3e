"""GPU vs the CPU oracle at the sizes the benchmark measures (all through the C ABI).

The kernels' launch shapes depend on the size of the problem: the far-field
pass has 63 block rows of 32 bodies at 2002 massive bodies (8 at 256), its
reduce adds 63 partials, the encounter task kernel sees ~150-190 encounter
bodies per step instead of a handful, the persistent sweep kernel cuts 4096
systems into items of a tuned grid, and the planetesimal disk splits 8196
sources over chunks.  These tests run the benchmarked workloads themselves:

- the 2002-body embryo disk (universal drift 100 steps from the initial
  conditions and 60 steps from the state after 320 steps, when ~190 bodies
  per step are in encounter; element drift 20 steps bit for bit), and the
  same disk with 300 eccentric embryos (the gated far-field pass);
- the 4096-system sweep (2.2 M bodies, 100 steps);
- the planetesimal disk (8196 massive bodies + 131072 test particles, 8 steps);
- the reference's Planet Nine sweep (32 systems x 10240 bodies), both drifts.

Tolerances as in test_gpu_parity.py: the element drift bit for bit with the
oracle's precision-2 mode (the GPU's elementary functions), the universal
drift at relative 1e-12 per body (positions and velocities); encounter flags,
encounter counts and drift-solve counts identical.
"""
import numpy as np
import pytest

import merc
import systems
from oracle import default_params as oparams
from test_gpu_parity import rel_err, run_both

pytestmark = pytest.mark.gpu

TOL = 1e-12


def check_universal(gs, st, op, ov, of, ost):
    assert rel_err(st.pos, op).max() <= TOL, rel_err(st.pos, op).max()
    assert rel_err(st.vel, ov).max() <= TOL, rel_err(st.vel, ov).max()
    assert np.array_equal(st.flags, of)
    assert gs.ce_body_steps == ost[0]
    assert gs.kepler_solves == ost[2]
    # pair sums that differ by ulps can move a Newton stop by one iteration
    assert abs(gs.kepler_iterations - ost[1]) <= max(2, ost[1] // 1000)


def test_embryo_disk_full_universal(oracle):
    sysm = systems.embryo_disk()
    assert sysm.n_total == 2002
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_UNIVERSAL)
    assert ost[0] > 100 * 100, "the disk should have >100 encounter bodies per step"
    check_universal(gs, st, op, ov, of, ost)


def test_embryo_disk_full_eccentric_partial_recompute(oracle):
    """300 of the 2002 embryos on e = 0.6 orbits: their far-field radius
    follows r_crit near pericentre, so at almost every step boundary some
    thresholds move and the gated far-field pass recomputes the block pairs
    of the blocks that moved, the second reduce taking each pair from the set
    it was last computed in.  Parity with the oracle at 1e-12 over 100 steps,
    and the same bits when the steps are split into calls (where the first
    kick of each call recomputes every pair)."""
    sysm = systems.embryo_disk()
    el = sysm.elements.reshape(6, -1)
    el[4, 2:2 + 300] = 0.6
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_UNIVERSAL)
    check_universal(gs, st, op, ov, of, ost)
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    a = merc.Integrator(merc.default_params(**kw))
    a.load_systems(sysm)
    a.step(40)
    assert a.far_recomputes() > 20
    b = merc.Integrator(merc.default_params(**kw))
    b.load_systems(sysm)
    for k in (3, 8, 29):
        b.step(k)
    assert np.array_equal(a.state().pos, b.state().pos) and np.array_equal(a.state().vel, b.state().vel)
    a.close()
    b.close()


def test_embryo_disk_full_universal_late_state(oracle):
    """The bench's timed region starts after 320 steps, where more bodies are
    in encounter than at the start: parity from that state (GPU-integrated,
    then given to both sides)."""
    sysm = systems.embryo_disk()
    kw = dict(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL)
    g = merc.Integrator(merc.default_params(**kw))
    g.load_systems(sysm)
    g.step(320)
    s0 = g.state()
    alag0 = g.a_lag()
    g.close()
    h = merc.Integrator(merc.default_params(**kw))
    h.load_state(sysm.body_offset, sysm.n_massive, sysm.mass, s0.pos, s0.vel, alag0)
    h.step(60)
    st, gs = h.state(), h.stats()
    h.close()
    op, ov, oal, of, ost = oracle.run(oparams(**kw), sysm.body_offset, sysm.n_massive, sysm.mass, s0.pos, s0.vel,
                                      alag0, steps=60, precision=2)
    assert ost[0] > 60 * 150, "the late state should have >150 encounter bodies per step"
    check_universal(gs, st, op, ov, of, ost)


def test_embryo_disk_full_elements_bitwise(oracle):
    sysm = systems.embryo_disk()
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 20, drift=merc.DRIFT_ELEMENTS)
    assert ost[0] > 0
    assert gs.ce_body_steps == ost[0]
    assert np.array_equal(st.flags, of)
    assert np.array_equal(st.pos, op), rel_err(st.pos, op).max()
    assert np.array_equal(st.vel, ov)
    assert np.array_equal(alag, oal)


def test_sweep_full_universal(oracle):
    sysm = systems.sweep()
    assert sysm.n_systems == 4096
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 100, drift=merc.DRIFT_UNIVERSAL)
    check_universal(gs, st, op, ov, of, ost)


def test_planetesimal_disk_full_universal(oracle):
    """8196 massive bodies + 131072 test particles, 8 steps: one full step
    graph (the test-particle half kicks merged across step boundaries)."""
    sysm = systems.planetesimal_disk()
    assert sysm.n_total == 8196 + 131072
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, 8, drift=merc.DRIFT_UNIVERSAL)
    check_universal(gs, st, op, ov, of, ost)


@pytest.mark.parametrize("drift", [merc.DRIFT_UNIVERSAL, merc.DRIFT_ELEMENTS])
def test_p9_sweep_full(oracle, drift):
    """The reference's own workload (examples/p9.json's layout: Planet Nine +
    4 giants + 10235 TNOs, 32 sweeps, dt 0.8219, changeover at 1 Hill radius)."""
    sysm = systems.p9_sweep()
    steps = 100 if drift == merc.DRIFT_UNIVERSAL else 20
    st, gs, alag, (op, ov, oal, of, ost) = run_both(oracle, sysm, steps, drift=drift)
    if drift == merc.DRIFT_UNIVERSAL:
        check_universal(gs, st, op, ov, of, ost)
    else:
        assert gs.ce_body_steps == ost[0]
        assert np.array_equal(st.flags, of)
        assert np.array_equal(st.pos, op, equal_nan=True), rel_err(st.pos, op).max()
        assert np.array_equal(st.vel, ov, equal_nan=True)
