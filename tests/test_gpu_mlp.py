"""Learned warm start: the hand-written GPU training kernels against the float64
numpy restatement (gradient check), and the end-to-end effect: a network
trained on the integrator's own logged drifts starts the FP64 Newton solve
closer to the root (fewer iterations) while the integration result stays the
same to 1e-12."""
import numpy as np
import pytest

import merc
import mlp_oracle
import systems

pytestmark = pytest.mark.gpu


def random_blob(rng):
    b = np.zeros(mlp_oracle.BLOB, np.float32)
    b[:mlp_oracle.NET] = rng.normal(0, 0.3, mlp_oracle.NET)
    b[mlp_oracle.IN_MEAN:mlp_oracle.IN_MEAN + 4] = [0.01, 1.0, 0.0, 0.0]
    b[mlp_oracle.IN_SCALE:mlp_oracle.IN_SCALE + 4] = [50.0, 2.0, 3.0, 1.0]
    b[mlp_oracle.OUT_MEAN] = 0.1
    b[mlp_oracle.OUT_SCALE] = 4.0
    b[mlp_oracle.BOX_LO:mlp_oracle.BOX_LO + 4] = [1e-5, 0.0, -2.0, -1.0]
    b[mlp_oracle.BOX_HI:mlp_oracle.BOX_HI + 4] = [0.1, 2.5, 2.0, 1.0]
    return b


def test_gradient_matches_cpu():
    rng = np.random.default_rng(5)
    blob = random_blob(rng)
    n = 300
    S = np.stack([rng.uniform(1e-4, 0.05, n), rng.uniform(0.5, 1.5, n), rng.uniform(-0.5, 0.5, n),
                  rng.choice([-1.0, 1.0], n), rng.normal(0.1, 0.3, n)], 1).astype(np.float32)
    loss, g = merc.mlp_grad(S, blob)
    loss_ref, g_ref = mlp_oracle.loss_and_grad(blob, S)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    err = np.abs(g - g_ref)
    assert err.max() <= 1e-4 * np.abs(g_ref).max() + 1e-7, err.max()


def test_inference_matches_cpu():
    rng = np.random.default_rng(6)
    blob = random_blob(rng)
    s = systems.embryo_disk(n_embryos=126)
    g = merc.Integrator(merc.default_params(dt=s.dt, hill_factor=3.0, drift=merc.DRIFT_UNIVERSAL))
    g.load_systems(s)
    st = g.state()
    g.close()
    guess, solved, its = merc.warm_start_probe(st.pos, st.vel, s.dt, blob)
    ref = mlp_oracle.guess(blob, st.pos, st.vel, s.dt)
    assert np.max(np.abs(guess - ref) / np.abs(ref)) < 1e-6


def run(sysm, steps, warm, weights=None, log=0):
    g = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=sysm.hill_factor, drift=merc.DRIFT_UNIVERSAL,
                                            warm_start=warm))
    g.load_systems(sysm)
    if weights is not None:
        g.mlp_set_weights(weights)
    if log:
        g.mlp_log(log)
    g.step(steps)
    return g


def test_trained_warm_start_cuts_iterations_and_keeps_results():
    train_sys = systems.embryo_disk(n_embryos=510, seed=21)
    g = run(train_sys, 40, merc.WARM_PLAIN, log=200_000)
    assert g.mlp_log_count() > 10_000
    loss = g.mlp_train(epochs=40, batch=2048, lr=3e-3, seed=3)
    assert loss[-1] < 0.2 * loss[0], loss
    w = g.mlp_weights()
    g.close()
    test_sys = systems.embryo_disk(n_embryos=254, seed=22)
    plain = run(test_sys, 60, merc.WARM_PLAIN)
    learned = run(test_sys, 60, merc.WARM_MLP, weights=w)
    sp, sl = plain.stats(), learned.stats()
    it_plain = sp.kepler_iterations / sp.kepler_solves
    it_learned = sl.kepler_iterations / sl.kepler_solves
    a, b = plain.state(), learned.state()
    rel = np.abs(a.pos - b.pos).reshape(3, -1).max(0) / np.linalg.norm(a.pos.reshape(3, -1), axis=0)
    print(f"mean Newton iterations: plain {it_plain:.3f}, learned {it_learned:.3f}, max rel pos diff {rel.max():.2e}")
    assert rel.max() <= 1e-12
    assert np.array_equal(a.flags, b.flags)
    assert it_learned < 0.8 * it_plain
    assert sl.kepler_nonconverged == 0
