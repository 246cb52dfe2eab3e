"""Planet Nine sweep configuration in the reference's JSON schema.

A restatement of the reference's generator (utils/sim_config.py:69-207,
p9_setup_config), seeded so that it is reproducible:

- 10235 massless TNOs with a linearly spaced in [150, 500) AU, e linearly
  spaced between 1 - 30/150 and 1 - 50/500 (perihelia 30 to 50 AU),
  inclination linearly spaced in [0, 25) deg, node, argument of perihelion and
  mean anomaly uniform in [0, 2 pi);
- Planet Nine (5 Earth masses, a 500 AU, e 0.25, i 20 deg, node 86 deg,
  argument of perihelion 138 deg, mean anomaly -176.2 deg) and the four giants
  with their J2000 elements;
- bodies ordered Planet Nine first, then by decreasing mass (the giants, then
  the TNOs);
- 32 sweeps of Planet Nine's elements: each parameter takes 32 linearly
  spaced values over its range, shuffled independently (mass 6.6 -1.7/+2.6
  Earth masses, a 500 -120/+170 AU, i 15.6 -5.4/+5.2 deg, e 0.26 +-0.1,
  longitude of perihelion 246.7 -13.4/+15.1 deg, node 96.9 -15.5/+17.3 deg),
  the argument of perihelion being the longitude of perihelion minus the node,
  mean anomaly 0.

mint replaces body 0's elements by sweep 4 d + k on device d (k < 4), with
mean anomaly 0 and body 0's mass unchanged.

    python p9-integrator_gb300/p9_config.py out.json [--seed S]
"""
import argparse
import json
import math

import numpy as np

M_EARTH = 3.00338e-06
NUM_TNOS = 640 * 16 - 5
DEG = math.pi / 180.0

# name, mass, a, e, i (deg), node (deg), argument of perihelion (deg)
GIANTS = [
    ("Neptune", 5.14855965e-5, 30.06896348, 0.00858587, 1.76917, 131.72169, -86.75034),
    ("Uranus", 4.36430044e-5, 19.19126393, 0.04716771, 0.76986, 74.22988, -96.73436),
    ("Saturn", 0.000285716656, 9.53707032, 0.05415060, 2.48446, 113.71504, -21.2831),
    ("Jupiter", 0.000954588, 5.20336301, 0.04839266, 1.30530, 100.55615, -85.8023),
]


def _body(name, mass, a, e, inc, node, peri, mean):
    return {"name": name, "mass": mass, "semi_major_axis": a, "eccentricity": e, "inclination": inc,
            "longitude_of_ascending_node": node, "argument_of_perihelion": peri, "mean_anomaly": mean}


def _spread(lo, hi, n, rng):
    """n linearly spaced values lo + k (hi - lo) / n, shuffled."""
    v = [lo + k * (hi - lo) / n for k in range(n)]
    rng.shuffle(v)
    return v


def p9_config(seed: int = 20261209, n_sweeps: int = 32) -> dict:
    rng = np.random.default_rng(seed)
    doc = {"sweeps": [], "bodies": []}
    ranges = [
        (6.6 - 1.7, 6.6 + 2.6, M_EARTH),          # mass
        (500.0 - 120.0, 500.0 + 170.0, 1.0),      # a
        (15.6 - 5.4, 15.6 + 5.2, DEG),            # i
        (0.26 - 0.1, 0.26 + 0.1, 1.0),            # e
        (246.7 - 13.4, 246.7 + 15.1, DEG),        # longitude of perihelion
        (96.9 - 15.5, 96.9 + 17.3, DEG),          # node
    ]
    cols = [_spread(lo * f, hi * f, n_sweeps, rng) for lo, hi, f in ranges]
    for k in range(n_sweeps):
        mass, a, inc, e, varpi, node = (c[k] for c in cols)
        doc["sweeps"].append(_body("Planet Nine", mass, a, e, inc, node, varpi - node, 0.0))
    bodies = [_body("Planet Nine", 5 * M_EARTH, 500.0, 0.25, 20 * DEG, 86 * DEG, 138 * DEG,
                    2 * math.pi - 176.2 * DEG)]
    for name, m, a, e, inc, node, peri in GIANTS:
        bodies.append(_body(name, m, a, e, inc * DEG, node * DEG, 2 * math.pi + peri * DEG, 0.0))
    a_sp, i_sp = (500.0 - 150.0) / NUM_TNOS, 25 * DEG / NUM_TNOS
    e_lo, e_hi = 1.0 - 30.0 / 150.0, 1.0 - 50.0 / 500.0
    e_sp = (e_hi - e_lo) / NUM_TNOS
    ang = rng.uniform(0.0, 2 * math.pi, (NUM_TNOS, 3))
    for i in range(NUM_TNOS):
        bodies.append(_body(f"TNO-{i}", 0.0, 150.0 + a_sp * i, e_lo + i * e_sp, i_sp * i, ang[i, 0], ang[i, 1],
                            ang[i, 2]))
    # Planet Nine first, the rest by decreasing mass (stable: TNOs keep their order)
    doc["bodies"] = [bodies[0]] + sorted(bodies[1:], key=lambda b: b["mass"], reverse=True)
    return doc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--seed", type=int, default=20261209)
    a = ap.parse_args()
    with open(a.out, "w") as f:
        json.dump(p9_config(a.seed), f, indent=1)


if __name__ == "__main__":
    main()
