"""The reference's own mercurius_solver kernel on the GPU (TEST INFRASTRUCTURE).

ctypes binding of baseline/_ref/refgpu/librefgpu.so (oracle/refgpu/prepare.py
writes the patched copy of the reference's kernel there, build() compiles it
with refgpu_driver.cu), and the two comparisons it serves:

- outer_padded(): the outer-solar-system workload padded with far massless
  bodies to 112 bodies (the reference's launch needs N % 16 == 0 and at most
  N/16 massive bodies), four sweeps with different angles;
- p9(): the first four systems of the Planet Nine sweep (10240 bodies).

Only tests and the measurement in __main__ use this module.
    python oracle/refgpu/refgpu.py     # on a GPU host: JSON with timings and differences
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "baseline", "_ref", "refgpu", "librefgpu.so")
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)


def available() -> bool:
    return os.path.exists(LIB)


class RefGPU:
    def __init__(self, path: str = LIB):
        L = C.CDLL(path)
        L.refgpu_run.argtypes = [C.c_int, C.c_int, C.c_int, _f64p, _f64p, C.c_double, C.c_long, C.c_int, _f64p, _f64p,
                                 _f32p, C.c_char_p, C.c_int]
        L.refgpu_run.restype = C.c_int
        L.refgpu_sweeps.restype = C.c_int
        self.L = L
        self.sweeps = L.refgpu_sweeps()

    def run(self, elements, masses, n_massive, dt, steps, launches=1, device=0):
        """elements: sweeps x 6 x n; returns (pos sweeps x 3 x n, elements
        sweeps x 6 x n, ms per launch)."""
        el = np.ascontiguousarray(elements, np.float64)
        S, six, n = el.shape
        assert S == self.sweeps and six == 6
        m = np.ascontiguousarray(masses, np.float64)
        pos = np.zeros((S, n, 3))
        out_el = np.zeros_like(el)
        ms = np.zeros(launches, np.float32)
        err = C.create_string_buffer(512)
        st = self.L.refgpu_run(device, n, int(n_massive), el.ctypes.data_as(_f64p), m.ctypes.data_as(_f64p), dt,
                               int(steps), int(launches), pos.ctypes.data_as(_f64p), out_el.ctypes.data_as(_f64p),
                               ms.ctypes.data_as(_f32p), err, 512)
        if st:
            raise RuntimeError(f"refgpu_run status {st}: {err.value.decode()}")
        return pos.transpose(0, 2, 1).copy(), out_el, ms


def _paths():
    for p in (os.path.join(ROOT, "p9-integrator_gb300"), os.path.dirname(HERE)):
        if p not in sys.path:
            sys.path.insert(0, p)


def outer_padded(n_sweeps=4):
    """Four outer-solar-system variants (seeds differ) padded to 112 bodies with
    7 massless bodies on wide orbits (a 3000-4000 AU) that no massive body
    approaches.  Returns (Systems batch of the four, elements sweeps x 6 x n)."""
    _paths()
    import systems

    blocks = []
    for k in range(n_sweeps):
        s = systems.outer_solar_system(seed=20261203 + k)
        rows = s.element_rows()
        rng = np.random.default_rng(77 + k)
        npad = 112 - s.n_total
        pad = np.stack([rng.uniform(0, 0.3, npad), rng.uniform(0, 2 * np.pi, npad), rng.uniform(0, 2 * np.pi, npad),
                        rng.uniform(0, 2 * np.pi, npad), rng.uniform(0.0, 0.1, npad),
                        rng.uniform(3000.0, 4000.0, npad)])
        blocks.append((np.concatenate([s.mass, np.zeros(npad)]), np.concatenate([rows, pad], axis=1),
                       int(s.n_massive[0])))
    batch = systems._pack(blocks, 0.5, 1.0, 100, "outer-solar-system padded to 112 bodies")
    el = np.stack([b[1] for b in blocks])
    return batch, el


def p9(n_sweeps=4):
    _paths()
    import systems

    full = systems.p9_sweep()
    batch = full.subset(range(n_sweeps))
    n = int(batch.body_offset[1])
    el = batch.element_rows().reshape(6, n_sweeps, n).transpose(1, 0, 2).copy()
    return batch, el


def rel_diff(a, b):
    """Max over bodies of |a - b| / |b| per body (positions 3 x n)."""
    a = a.reshape(3, -1)
    b = b.reshape(3, -1)
    ok = np.isfinite(a).all(0) & np.isfinite(b).all(0)
    d = np.max(np.abs(a[:, ok] - b[:, ok]), axis=0) / np.linalg.norm(b[:, ok], axis=0)
    return float(d.max()), float(np.median(d)), int((~ok).sum())


def compare(batch, el, steps, dt, hill_factor, compat_block, launches=1, time_launches=0):
    """The reference kernel, this library's element and universal paths and the
    oracle on the same systems; returns a dict of differences and timings."""
    _paths()
    import merc
    from oracle import Oracle
    from oracle import default_params as oparams

    R = RefGPU()
    S = R.sweeps
    n = int(batch.body_offset[1])
    nm = int(batch.n_massive[0])
    masses = batch.mass[:n]
    rpos, rel_, ms = R.run(el, masses, nm, dt, steps, launches)
    ref_pos = np.concatenate([rpos[s] for s in range(S)], axis=1)  # 3 x (S n)
    out = {"n_bodies": n, "n_massive": nm, "sweeps": S, "steps": steps * launches, "dt": dt}
    kw = dict(dt=dt, hill_factor=hill_factor, compat_block=compat_block)
    res = {}
    for name, drift in (("elements", merc.DRIFT_ELEMENTS), ("universal", merc.DRIFT_UNIVERSAL)):
        g = merc.Integrator(merc.default_params(drift=drift, **kw))
        g.load_systems(batch)
        for k in range(launches):
            if k and drift == merc.DRIFT_ELEMENTS:
                g.roundtrip()  # the reference restarts every launch from elements
            g.step(steps)
        res[name] = g.state().pos.reshape(3, -1)
        g.close()
    O = Oracle()
    p = oparams(drift=0, **kw)
    pos, vel, al = O.load_elements(p, batch.body_offset, batch.n_massive, batch.mass, batch.elements, precision=0)
    for k in range(launches):
        if k:
            pos, vel, al = O.roundtrip(p, batch.body_offset, batch.n_massive, batch.mass, pos, vel, precision=0)
        pos, vel, al, fl, _st = O.run(p, batch.body_offset, batch.n_massive, batch.mass, pos, vel, al, steps=steps,
                                      precision=0)
    oracle_pos = pos.reshape(3, -1)
    out["ours_elements_vs_reference_gpu"] = rel_diff(res["elements"], ref_pos)
    out["oracle_host_libm_vs_reference_gpu"] = rel_diff(oracle_pos, ref_pos)
    out["ours_elements_vs_oracle_host_libm"] = rel_diff(res["elements"], oracle_pos)
    out["ours_universal_vs_reference_gpu"] = rel_diff(res["universal"], ref_pos)
    if time_launches:
        _, _, tms = R.run(el, masses, nm, dt, steps, time_launches)
        t = float(np.median(tms[1:] if len(tms) > 1 else tms))
        out["reference_gpu_ms_per_step"] = t / steps
        out["reference_gpu_body_steps_per_s"] = S * n * steps / (t * 1e-3)
        for name, drift in (("elements", merc.DRIFT_ELEMENTS), ("universal", merc.DRIFT_UNIVERSAL)):
            g = merc.Integrator(merc.default_params(drift=drift, **kw))
            g.load_systems(batch)
            g.step(2)
            g.step(steps)
            t2 = g.stats().last_step_ms
            g.close()
            out[f"ours_{name}_ms_per_step"] = t2 / steps
            out[f"ours_{name}_body_steps_per_s"] = S * n * steps / (t2 * 1e-3)
    return out


def main():
    res = {}
    batch, el = outer_padded()
    res["outer_padded"] = compare(batch, el, 100, 0.5, 1.0, 7, time_launches=4)
    res["outer_padded_2_launches"] = compare(batch, el, 50, 0.5, 1.0, 7, launches=2)
    batch, el = p9()
    res["p9_4_sweeps"] = compare(batch, el, 100, 0.8219, 1.0, 640, time_launches=4)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
