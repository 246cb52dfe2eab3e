"""Checkpoint/resume and the per-system loader.

- merc_save_checkpoint / merc_load_checkpoint: a restored context continues
  with the same bits as the saved one (state, flags, counters, warm-start
  network), and damaged files are rejected;
- mint --checkpoint / --resume: a run resumed from the checkpoint of its
  first batch ends in a byte-identical checkpoint to the uninterrupted run;
- merc_load_systems equals merc_load_elements / merc_load_state of the
  concatenated arrays."""
import os
import subprocess

import numpy as np
import pytest

import merc
import systems

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MINT = os.path.join(ROOT, "p9-integrator_gb300", "mint", "mint")


@pytest.mark.parametrize("drift", [merc.DRIFT_UNIVERSAL, merc.DRIFT_ELEMENTS])
def test_checkpoint_resume_is_exact(tmp_path, drift):
    sysm = systems.concat([systems.embryo_disk(n_embryos=60, seed=3), systems.outer_solar_system(n_test=20)])
    kw = dict(dt=0.01, hill_factor=3.0, drift=drift)
    a = merc.Integrator(merc.default_params(**kw))
    a.load_systems(sysm)
    a.step(11)
    ck = tmp_path / "state.ckpt"
    a.save_checkpoint(ck)
    a.step(13)
    sa, ta = a.state(), a.stats()
    b = merc.Integrator(merc.default_params())  # parameters come from the file
    b.load_checkpoint(ck)
    assert b.stats().steps_done == 11
    b.step(13)
    sb, tb = b.state(), b.stats()
    assert np.array_equal(sa.pos, sb.pos) and np.array_equal(sa.vel, sb.vel)
    assert np.array_equal(sa.flags, sb.flags)
    assert (ta.steps_done, ta.ce_body_steps, ta.kepler_iterations) == (tb.steps_done, tb.ce_body_steps,
                                                                       tb.kepler_iterations)
    a.close()
    b.close()


def test_checkpoint_keeps_the_warm_start_network(tmp_path):
    sysm = systems.outer_solar_system(n_test=40)
    g = merc.Integrator(merc.default_params(dt=sysm.dt, hill_factor=3.0, drift=merc.DRIFT_UNIVERSAL))
    g.load_systems(sysm)
    w = np.random.default_rng(1).normal(0, 0.01, merc.MLP_BLOB).astype(np.float32)
    w[-18:] = [0, 0, 0, 0, 1, 1, 1, 1, 0, 1, -1e30, -1e30, -1e30, -1e30, 1e30, 1e30, 1e30, 1e30]
    g.mlp_set_weights(w)
    ck = tmp_path / "m.ckpt"
    g.save_checkpoint(ck)
    h = merc.Integrator(merc.default_params())
    h.load_checkpoint(ck)
    assert np.array_equal(h.mlp_weights(), w)
    g.close()
    h.close()


def test_damaged_checkpoint_is_rejected(tmp_path):
    sysm = systems.outer_solar_system(n_test=5)
    g = merc.Integrator(merc.default_params(dt=0.5, drift=merc.DRIFT_UNIVERSAL))
    g.load_systems(sysm)
    ck = tmp_path / "c.ckpt"
    g.save_checkpoint(ck)
    raw = bytearray(ck.read_bytes())
    raw[200] ^= 1
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(bytes(raw))
    (tmp_path / "short.ckpt").write_bytes(bytes(raw[:100]))
    h = merc.Integrator(merc.default_params())
    for f in (bad, tmp_path / "short.ckpt", tmp_path / "missing.ckpt"):
        with pytest.raises(merc.MercError) as e:
            h.load_checkpoint(f)
        assert e.value.code == merc.MERC_ERR_CONFIG
    g.close()
    h.close()


def test_load_systems_equals_concatenated_load():
    sysm = systems.sweep(n_systems=5, nt_lo=10, nt_hi=60, seed=21)
    rows = sysm.element_rows()
    descs = []
    for s in range(sysm.n_systems):
        b0, b1 = sysm.body_offset[s], sysm.body_offset[s + 1]
        descs.append({"n_massive": int(sysm.n_massive[s]), "mass": sysm.mass[b0:b1], "elements": rows[:, b0:b1]})
    kw = dict(dt=sysm.dt, hill_factor=3.0, drift=merc.DRIFT_UNIVERSAL)
    a = merc.Integrator(merc.default_params(**kw))
    a.load_systems(sysm)
    b = merc.Integrator(merc.default_params(**kw))
    b.load_system_list(descs)
    a.step(7)
    b.step(7)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa.pos, sb.pos) and np.array_equal(sa.vel, sb.vel)
    # by state: descriptors with pos/vel give the same as merc_load_state
    pos, vel = sa.pos.reshape(3, -1), sa.vel.reshape(3, -1)
    descs2 = [{"n_massive": d["n_massive"], "mass": d["mass"],
               "pos": pos[:, sysm.body_offset[s]:sysm.body_offset[s + 1]],
               "vel": vel[:, sysm.body_offset[s]:sysm.body_offset[s + 1]]} for s, d in enumerate(descs)]
    c = merc.Integrator(merc.default_params(**kw))
    c.load_system_list(descs2)
    d = merc.Integrator(merc.default_params(**kw))
    d.load_state(sysm.body_offset, sysm.n_massive, sysm.mass, sa.pos, sa.vel)
    c.step(5)
    d.step(5)
    assert np.array_equal(c.state().pos, d.state().pos) and np.array_equal(c.state().vel, d.state().vel)
    for g in (a, b, c, d):
        g.close()


@pytest.mark.skipif(not os.path.exists(MINT), reason="mint not built")
def test_mint_resume_matches_uninterrupted_run(tmp_path):
    s = systems.outer_solar_system(n_test=11)
    cfg = tmp_path / "c.json"
    systems.to_json(s, str(cfg), dt=0.5, batch_size=15, changeover_hill_factor=3.0, drift="universal")

    def run(*args):
        out = subprocess.run([MINT, "-c", str(cfg), *args], capture_output=True, text=True, cwd=tmp_path)
        assert out.returncode == 0, out.stderr

    run("-t", "3", "--checkpoint", "full.ckpt")
    run("-t", "1", "--checkpoint", "first.ckpt")
    run("-t", "3", "--resume", "first.ckpt", "--checkpoint", "resumed.ckpt")
    assert (tmp_path / "full.ckpt").read_bytes() == (tmp_path / "resumed.ckpt").read_bytes()
