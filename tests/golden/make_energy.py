"""Generate the energy fixtures: energy after 1e4 steps from the CPU oracle in
long double (the energy-error reference) and in binary64, with the
reference's element drift (the reference algorithm) and the universal drift.

    python tests/golden/make_energy.py outer    -> energy_outer.json
        outer-solar-system workload (5 massive bodies + 100 test particles,
        dt 0.5 yr, changeover 3 Hill radii)
    python tests/golden/make_energy.py embryo   -> energy_embryo.json
        the 2002-body embryo disk (dt 0.01 yr, changeover 3 Hill radii, close
        encounters every step): binary64 over 1e4 steps (energies after 300
        and after 1e4 steps), long double over the first 300 steps only (the
        host's long-double fma is a software routine, ~130x slower than
        binary64: 1e4 steps would take ~10 hours on 8 cores); ~40 minutes

Run from the repository root.
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "p9-integrator_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import systems  # noqa: E402
from oracle import Oracle, build  # noqa: E402
from oracle import default_params as oparams  # noqa: E402

STEPS = 10000


EMBRYO_SHORT = 300


def main_embryo():
    build()
    O = Oracle()
    s = systems.embryo_disk()
    out = {"workload": s.label, "steps": STEPS, "short_steps": EMBRYO_SHORT, "dt": s.dt,
           "hill_factor": s.hill_factor}
    for drift, name in ((0, "elements"), (1, "universal")):
        p = oparams(dt=s.dt, hill_factor=s.hill_factor, drift=drift)
        pos, vel, alag = O.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements)
        e0 = float(O.energy(s.body_offset, s.n_massive, s.mass, pos, vel)[0])
        t = time.time()
        res = {"energy0": e0}
        a, b, al, fl, _ = O.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=EMBRYO_SHORT)
        e1 = float(O.energy(s.body_offset, s.n_massive, s.mass, a, b)[0])
        a, b, *_ = O.run(p, s.body_offset, s.n_massive, s.mass, a, b, al, flags=fl, steps=STEPS - EMBRYO_SHORT)
        e2 = float(O.energy(s.body_offset, s.n_massive, s.mass, a, b)[0])
        res["binary64"] = {"energy_short": e1, "rel_error_short": abs(e1 - e0) / abs(e0), "energy": e2,
                           "rel_error": abs(e2 - e0) / abs(e0)}
        if drift == 1:
            a, b, *_ = O.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=EMBRYO_SHORT, precision=1)
            e1 = float(O.energy(s.body_offset, s.n_massive, s.mass, a, b)[0])
            res["long_double"] = {"energy_short": e1, "rel_error_short": abs(e1 - e0) / abs(e0)}
        out[name] = res
        print(name, res, f"{time.time() - t:.1f}s", flush=True)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "energy_embryo.json"), "w") as f:
        json.dump(out, f, indent=1)


def main(which="outer"):
    if which == "embryo":
        return main_embryo()
    build()
    O = Oracle()
    s = systems.outer_solar_system() if which == "outer" else systems.embryo_disk()
    out = {"workload": s.label, "steps": STEPS, "dt": s.dt, "hill_factor": s.hill_factor}
    for drift, name in ((0, "elements"), (1, "universal")):
        p = oparams(dt=s.dt, hill_factor=s.hill_factor, drift=drift)
        pos, vel, alag = O.load_elements(p, s.body_offset, s.n_massive, s.mass, s.elements)
        e0 = float(O.energy(s.body_offset, s.n_massive, s.mass, pos, vel)[0])
        t = time.time()
        res = {}
        for prec, tag in ((0, "binary64"), (1, "long_double")):
            a, b, *_ = O.run(p, s.body_offset, s.n_massive, s.mass, pos, vel, alag, steps=STEPS, precision=prec)
            e1 = float(O.energy(s.body_offset, s.n_massive, s.mass, a, b)[0])
            res[tag] = {"energy": e1, "rel_error": abs(e1 - e0) / abs(e0)}
        out[name] = {"energy0": e0, **res}
        print(name, res, f"{time.time() - t:.1f}s")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), f"energy_{which}.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "outer")
