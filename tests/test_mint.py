"""The drop-in mint CLI: argument and config handling (CPU) and a short GPU run
checked against the oracle (same batch structure: steps, then the reference's
element round trip at every batch boundary)."""
import os
import subprocess

import numpy as np
import pytest

import systems
from oracle import default_params as oparams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MINT = os.path.join(ROOT, "p9-integrator_gb300", "mint", "mint")


def have_mint():
    return os.path.exists(MINT)


@pytest.mark.skipif(not have_mint(), reason="mint not built")
def test_dry_run_prints_the_system(tmp_path):
    s = systems.outer_solar_system(n_test=3)
    cfg = tmp_path / "c.json"
    systems.to_json(s, str(cfg), dt=0.5, batch_size=10)
    out = subprocess.run([MINT, "-c", str(cfg), "-t", "3", "--dry-run"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert "Simulation with 8 bodies" in out.stdout
    assert "batch 10 steps x 3 batches" in out.stdout


@pytest.mark.skipif(not have_mint(), reason="mint not built")
def test_rejects_missing_config_and_bad_drift(tmp_path):
    out = subprocess.run([MINT, "-t", "1"], capture_output=True, text=True)
    assert out.returncode != 0 and "no config" in out.stderr
    s = systems.outer_solar_system(n_test=3)
    cfg = tmp_path / "c.json"
    systems.to_json(s, str(cfg), drift="leapfrog")
    out = subprocess.run([MINT, "-c", str(cfg), "--dry-run"], capture_output=True, text=True)
    assert out.returncode != 0 and "unknown drift" in out.stderr


@pytest.mark.gpu
def test_mint_run_matches_oracle(tmp_path, oracle):
    s = systems.outer_solar_system(n_test=11)
    cfg = tmp_path / "c.json"
    systems.to_json(s, str(cfg), dt=0.5, batch_size=25, changeover_hill_factor=3.0)
    out = subprocess.run([MINT, "-c", str(cfg), "-t", "2", "-o", str(tmp_path / "pos.txt"), "--dump-precise",
                          str(tmp_path / "precise.txt")], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    assert "NaN counter for  1 timestep (mYrs): 0" in out.stdout
    blocks = open(tmp_path / "precise.txt").read().split("#\n")[1:]
    assert len(blocks) == 1  # batch 0 only: checkpoints every 20 batches
    got = np.array([[float(v) for v in ln.split()] for ln in blocks[0].split("$\n")[1].strip().splitlines()])
    p = oparams(dt=0.5, hill_factor=3.0)
    pos, vel, alag = oracle.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements, precision=2)
    op, ov, _, _, _ = oracle.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=25, precision=2)
    assert np.array_equal(got.T.reshape(-1), op)
    # the 6-digit positions file has the reference layout
    txt = open(tmp_path / "pos.txt").read().splitlines()
    assert txt[0] == "#" and txt[1] == "$" and len(txt[2].split()) == 3


@pytest.mark.gpu
def test_mint_radius_key_turns_collisions_on(tmp_path):
    """A per-body "radius" key in the config switches physical collisions on
    (merc_set_radii): the accretion case of test_collisions.py, run through
    mint, reports its one collision."""
    from test_collisions import accretion_case

    s, rad = accretion_case()
    cfg = tmp_path / "c.json"
    systems.to_json(s, str(cfg), dt=s.dt, batch_size=5, changeover_hill_factor=3.0)
    import json

    doc = json.load(open(cfg))
    for b, r in zip(doc["bodies"], rad):
        b["radius"] = float(r)
    json.dump(doc, open(cfg, "w"))
    out = subprocess.run([MINT, "-c", str(cfg), "-t", "2", "-i", "-o", str(tmp_path / "pos.txt")],
                         capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    assert "Collisions: 1" in out.stdout
