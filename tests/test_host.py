"""Host-side checks that need no GPU: the C ABI library loads and exports every
function its headers declare, parameter validation, the workload generators
and the JSON system-config format."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

import systems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "p9-integrator_gb300", "libmerc.so")

def _ref_examples():
    from oracle import ref_dir

    d = ref_dir()
    return os.path.join(d, "examples") if d else None


REF_EXAMPLES = _ref_examples()


@pytest.fixture(scope="module")
def libmerc():
    if not os.path.exists(LIB):
        import __graft_entry__  # noqa: F401

        pytest.skip("libmerc.so not built")
    return C.CDLL(LIB)


def declared_functions():
    names = []
    for h in ("merc.h", "merc_diag.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(merc_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(libmerc):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(libmerc, n), n


def test_default_params_are_the_reference_constants(libmerc):
    import merc

    p = merc.default_params()
    assert p.dt == 0.8219 and p.softening2 == 1e-8 and p.hill_factor == 1.0
    assert p.kepler_iters == 8 and p.bs_rows == 3 and p.kepler_tol == 1e-13


def test_create_rejects_bad_params_before_touching_a_device(libmerc):
    import merc

    for kw in (dict(dt=0.0), dict(bs_rows=5), dict(kepler_iters=0), dict(drift=7), dict(softening2=2.0),
               dict(compat_block=-1), dict(kepler_max_iter=0)):
        p = merc.default_params(**kw)
        h = C.c_void_p()
        assert merc.lib().merc_create(0, C.byref(p), C.byref(h)) == merc.MERC_ERR_CONFIG, kw


def test_step_static_validates_without_a_device(libmerc):
    import merc

    L = merc.lib()
    p = merc.default_params(drift=merc.DRIFT_UNIVERSAL)
    one = C.c_void_p(8)
    assert L.merc_step_static(0, C.byref(p), 0, 0, one, one, one, None, 1, None) == merc.MERC_ERR_CONFIG
    assert L.merc_step_static(0, C.byref(p), 4, 5, one, one, one, None, 1, None) == merc.MERC_ERR_CONFIG
    assert L.merc_step_static(0, None, 4, 1, one, one, one, None, 1, None) == merc.MERC_ERR_CONFIG


def test_workload_shapes():
    s0 = systems.outer_solar_system()
    assert s0.n_total == 105 and int(s0.n_massive[0]) == 5 and s0.dt == 0.5 and s0.hill_factor == 3.0
    el = s0.element_rows()
    a, e = el[5], el[4]
    q = a[5:] * (1 - e[5:])
    assert np.all((q >= 30) & (q <= 50)) and np.all((a[5:] >= 150) & (a[5:] <= 1000))
    assert np.all(s0.mass[5:] == 0) and np.all(s0.mass[:5] > 1e-12)
    s1 = systems.embryo_disk()
    assert s1.n_total == 2002 and int(s1.n_massive[0]) == 2002
    emb = s1.element_rows()[5][2:]
    assert emb.min() >= 0.5 and emb.max() <= 1.5
    # surface density ~ a^-1.5  ->  sqrt(a) uniform
    assert abs(np.mean(np.sqrt(emb)) - 0.5 * (np.sqrt(0.5) + np.sqrt(1.5))) < 0.01
    m = s1.mass[2:] / systems.M_EARTH
    assert m.min() >= 0.025 and m.max() <= 0.1
    s2 = systems.sweep(n_systems=64)
    nt = s2.sizes() - 5
    assert nt.min() >= 64 and nt.max() <= 1024 and np.all(s2.n_massive == 5)
    assert s2.pairs_per_step() == int(2 * np.sum(5 * 4 + nt * 5))


def test_seeded_generators_are_reproducible():
    a = systems.sweep(n_systems=8, seed=3)
    b = systems.sweep(n_systems=8, seed=3)
    assert np.array_equal(a.elements, b.elements) and np.array_equal(a.body_offset, b.body_offset)


def test_json_round_trip(tmp_path):
    s = systems.outer_solar_system(n_test=7)
    path = tmp_path / "sys.json"
    systems.to_json(s, str(path), dt=0.5)
    d = systems.from_json(str(path))
    assert np.array_equal(d["mass"], s.mass)
    assert np.array_equal(d["elements"].reshape(-1), s.elements)
    assert d["options"]["dt"] == 0.5
    assert systems.count_massive(d["mass"]) == 5


@pytest.mark.skipif(not REF_EXAMPLES or not os.path.isdir(REF_EXAMPLES), reason="reference examples not present")
def test_reference_example_configs_parse():
    for name in ("earth_and_mars.json", "planetary_embryos.json", "p9.json"):
        d = systems.from_json(os.path.join(REF_EXAMPLES, name))
        assert d["elements"].shape[0] == 6 and d["mass"].size == d["elements"].shape[1]
    p9 = systems.from_json(os.path.join(REF_EXAMPLES, "p9.json"))
    assert p9["mass"].size == 10240 and len(p9["sweeps"]) == 32
    assert systems.count_massive(p9["mass"]) == 5
