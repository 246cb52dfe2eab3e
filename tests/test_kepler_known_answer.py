"""Known-answer tests independent of the reference: with no massive bodies the
step is a pure two-body drift, so positions after 100 steps must equal the
closed-form ellipse (Kepler's equation solved to convergence in float64).
The universal drift (oracle and GPU) meets 1e-12 per body (measured 2e-15
in positions).  The element drift is the reference's algorithm, whose element
conversion adds 1e-8 to h^2 (sim.cuh:250); for near-circular orbits that
moves e by ~1e-8 / e per step, and after 100 steps the reference's own code
(oracle, pinned bit for bit to it) is 3e-5 away from the ellipse in position
and 1.2e-4 in velocity.  The GPU element path is held to the oracle bit for
bit and to 1e-3 of the ellipse."""
import numpy as np
import pytest

import kepler_closed_form as kc
from oracle import default_params as oparams

DT, STEPS = 0.01, 100


def rel(a, b):
    a, b = a.reshape(3, -1), b.reshape(3, -1)
    return np.max(np.abs(a - b), axis=0) / np.linalg.norm(b, axis=0)


def test_oracle_universal_drift_matches_closed_form(oracle):
    off, nm, m, el = kc.test_particle_batch()
    p = oparams(dt=DT, hill_factor=3.0, drift=1)
    pos, vel, al = oracle.load_elements(p, off, nm, m, el.reshape(-1))
    p0, v0 = kc.state(el, 0.0)
    assert rel(pos, p0).max() < 1e-14 and rel(vel, v0).max() < 1e-14
    op, ov, _, fl, _ = oracle.run(p, off, nm, m, pos, vel, al, steps=STEPS)
    pt, vt = kc.state(el, DT * STEPS)
    assert rel(op, pt).max() <= 1e-12
    assert rel(ov, vt).max() <= 1e-12
    assert not np.any(fl & 1)


@pytest.mark.gpu
@pytest.mark.parametrize("drift,tol", [(1, 1e-12), (0, 1e-3)])
def test_gpu_drift_matches_closed_form(oracle, drift, tol):
    import merc

    off, nm, m, el = kc.test_particle_batch()
    g = merc.Integrator(merc.default_params(dt=DT, hill_factor=3.0, drift=drift))
    g.load_elements(off, nm, m, el.reshape(-1))
    g.step(37)
    g.step(STEPS - 37)
    st = g.state()
    g.close()
    pt, vt = kc.state(el, DT * STEPS)
    assert rel(st.pos, pt).max() <= tol
    assert rel(st.vel, vt).max() <= tol
    assert not np.any(st.flags & 1)
    if drift == 0:
        p = oparams(dt=DT, hill_factor=3.0, drift=0)
        pos, vel, al = oracle.load_elements(p, off, nm, m, el.reshape(-1), precision=2)
        op, ov, _, _, _ = oracle.run(p, off, nm, m, pos, vel, al, steps=STEPS, precision=2)
        assert np.array_equal(st.pos, op) and np.array_equal(st.vel, ov)
