"""Generate the golden vectors of tests/golden from the reference's own code.

Runs the reference's src/sim.cuh compiled for the host (oracle/_ref/librefhost.so,
built by `make -C oracle ref` where the reference sources are present) on small
seeded inputs and stores inputs and outputs as JSON (floats round-trip exactly).
Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "p9-integrator_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import systems  # noqa: E402
from oracle import RefHost, build  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def padded_outer(n_total=112, seed=20261203):
    s = systems.outer_solar_system(seed=seed)
    pad = n_total - s.n_total
    el = s.element_rows()
    padel = np.stack([np.zeros(pad), np.zeros(pad), np.zeros(pad), np.linspace(0, 6, pad), np.full(pad, 0.1),
                      np.linspace(2000, 3000, pad)])
    return np.concatenate([el, padel], axis=1), np.concatenate([s.mass, np.zeros(pad)]), int(s.n_massive[0])


def main():
    build()
    R = RefHost()
    cases = []

    def add(name, el, m, nm, block, dt, hill, steps):
        rp, rv, ra, _, ce = R.run(el.reshape(-1), m, nm, block, dt, hill, steps)
        cases.append({"name": name, "elements": el.reshape(-1).tolist(), "mass": m.tolist(), "n_massive": nm,
                      "block": block, "dt": dt, "hill_factor": hill, "steps": steps, "pos": rp.tolist(),
                      "vel": rv.tolist(), "a_lag": ra.tolist(), "ce_last": ce.astype(int).tolist()})

    el, m, nm = padded_outer()
    add("outer-solar-system padded to 112, one block", el, m, nm, 112, 0.5, 3.0, 40)
    add("outer-solar-system padded to 112, blocks of 7 (threadIdx quirk)", el, m, nm, 7, 0.5, 3.0, 40)
    s = systems.embryo_disk(n_embryos=62, seed=5)
    add("embryo disk, 64 massive bodies, encounters", s.element_rows(), s.mass, 64, 64, 0.01, 3.0, 40)
    s = systems.sweep(n_systems=1, nt_lo=59, nt_hi=59, seed=6)
    add("sweep system, 5 massive + 59 test particles, reference changeover", s.element_rows(), s.mass, 5, 64, 0.8219,
        1.0, 40)
    with open(os.path.join(OUT, "reference_runs.json"), "w") as f:
        json.dump({"source": "reference src/sim.cuh compiled for the host (oracle/_ref)", "cases": cases}, f)

    rng = np.random.default_rng(17)
    n = 400
    M = rng.uniform(0, 2 * np.pi, n)
    e = np.concatenate([rng.uniform(0, 0.99, n - 40), rng.uniform(1.01, 3.0, 40)])
    E = R.danby(M, e)
    el = np.stack([rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n), M,
                   rng.uniform(0, 0.95, n), rng.uniform(0.3, 1000, n)]).reshape(-1)
    pos, vel = R.cart_from_elem(el)
    back = R.elem_from_cart(pos, vel)
    with open(os.path.join(OUT, "reference_units.json"), "w") as f:
        json.dump({"source": "reference src/sim.cuh compiled for the host (oracle/_ref)", "danby_M": M.tolist(),
                   "danby_e": e.tolist(), "danby_E": E.tolist(), "elements": el.tolist(), "pos": pos.tolist(),
                   "vel": vel.tolist(), "elements_back": back.tolist()}, f)
    print("wrote", len(cases), "run cases and unit vectors")


if __name__ == "__main__":
    main()
