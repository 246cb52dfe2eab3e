"""The Planet Nine sweep configuration (p9_config.py, restating the
reference's generator utils/sim_config.py:69-207) and mint reading it.

The deterministic fields (body order, masses, the giants' and Planet Nine's
elements, the TNOs' a, e and i sequences, the sweep grids) are compared with
the reference's own examples/p9.json where the reference sources are present;
the random angles are drawn from a seed here and are not compared."""
import json
import os
import subprocess

import numpy as np
import pytest

import p9_config
import systems

from oracle import ref_dir

REF = os.path.join(ref_dir(), "examples", "p9.json") if ref_dir() else None
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MINT = os.path.join(ROOT, "p9-integrator_gb300", "mint", "mint")
FIXED = ["mass", "semi_major_axis", "eccentricity", "inclination"]


def test_structure():
    d = p9_config.p9_config()
    b = d["bodies"]
    assert len(b) == 10240 and len(d["sweeps"]) == 32
    assert [x["name"] for x in b[:5]] == ["Planet Nine", "Jupiter", "Saturn", "Neptune", "Uranus"]
    a = np.array([x["semi_major_axis"] for x in b[5:]])
    e = np.array([x["eccentricity"] for x in b[5:]])
    q = a * (1 - e)
    assert np.all(np.diff(a) > 0) and a[0] == 150.0 and a[-1] < 500.0
    # perihelia run from 30 AU to 50 AU at the ends (a and e are spaced
    # linearly and independently, so q is not monotonic in between)
    assert q[0] == pytest.approx(30.0, rel=1e-12) and q[-1] == pytest.approx(50.0, rel=1e-3)
    sw = d["sweeps"]
    for key, lo, hi in [("semi_major_axis", 380.0, 670.0), ("eccentricity", 0.16, 0.36)]:
        v = np.sort([s[key] for s in sw])
        assert np.allclose(v, lo + np.arange(32) * (hi - lo) / 32)
    s = systems.p9_sweep()
    assert s.n_systems == 32 and s.n_total == 32 * 10240 and set(s.n_massive) == {5}


@pytest.mark.skipif(not REF or not os.path.exists(REF), reason="reference examples not present on this host")
def test_deterministic_fields_equal_the_reference_example():
    ref = json.load(open(REF))
    mine = p9_config.p9_config()
    assert len(ref["bodies"]) == len(mine["bodies"])
    for rb, mb in zip(ref["bodies"], mine["bodies"]):
        assert rb["name"] == mb["name"]
        for k in FIXED:
            assert rb[k] == pytest.approx(mb[k], rel=1e-15, abs=1e-300), (rb["name"], k)
    for k in ("longitude_of_ascending_node", "argument_of_perihelion", "mean_anomaly"):
        for j in range(5):  # the planets' angles are fixed numbers
            assert ref["bodies"][j][k] == pytest.approx(mine["bodies"][j][k], rel=1e-15)
    # sweep grids: the same sets of values per parameter (order is a shuffle)
    for k in ("mass", "semi_major_axis", "inclination", "eccentricity"):
        assert np.allclose(np.sort([s[k] for s in ref["sweeps"]]), np.sort([s[k] for s in mine["sweeps"]]),
                           rtol=1e-14, atol=0)


@pytest.mark.skipif(not os.path.exists(MINT), reason="mint not built")
def test_mint_reads_the_p9_config(tmp_path):
    cfg = tmp_path / "p9.json"
    with open(cfg, "w") as f:
        json.dump(p9_config.p9_config(), f)
    for dev, first in ((0, 0), (7, 28)):
        out = subprocess.run([MINT, "-c", str(cfg), "-t", "1", "-d", str(dev), "--dry-run"], capture_output=True,
                             text=True)
        assert out.returncode == 0, out.stderr
        assert "Systems: 4 x 10240 bodies (5 massive)" in out.stdout
    out = subprocess.run([MINT, "-c", str(cfg), "-t", "1", "-d", "8", "--dry-run"], capture_output=True, text=True)
    assert out.returncode != 0 and "needs sweep 32" in out.stderr
