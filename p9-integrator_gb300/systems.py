"""Planetary systems: seeded generators of the benchmark workloads and the
reference's JSON system-config format.

Units: G = 1, M_sun = 1 (implicit, at the origin), AU, yr, angles in radians.
Bodies are ordered massive first, the order the reference assumes when it
counts massive bodies (src/mercurius.cu:4-15) and loops over the first Nm
(src/sim.cuh:339).

Element arrays are 6 x n in the order inclination, longitude of ascending
node, argument of perihelion, mean anomaly, eccentricity, semi-major axis
(the order of merc_load_elements in include/merc.h).

The generators stand in for the reference's offline config tool
(utils/sim_config.py), which writes examples/p9.json: they draw the five
benchmark workloads from a seed with the documented distributions.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

M_EARTH = 3.0e-6
DEG = np.pi / 180.0
TWO_PI = 2.0 * np.pi
# outer-solar-system analogue: (mass, semi-major axis) of the four giants
GIANTS = [(9.55e-4, 5.20), (2.86e-4, 9.58), (4.37e-5, 19.2), (5.15e-5, 30.1)]
MASSIVE_THRESHOLD = 1e-12  # src/mercurius.cu:9

ELEMENT_KEYS = ["inclination", "longitude_of_ascending_node", "argument_of_perihelion", "mean_anomaly",
                "eccentricity", "semi_major_axis"]


@dataclass
class Systems:
    """A batch of independent systems, concatenated body-wise."""

    body_offset: np.ndarray  # int64, n_systems + 1
    n_massive: np.ndarray  # int32, n_systems
    mass: np.ndarray  # float64, n_total
    elements: np.ndarray  # float64, 6 x n_total (flattened row-major)
    dt: float = 0.5
    hill_factor: float = 3.0
    steps: int = 10000
    names: Optional[List[str]] = None
    label: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n_systems(self) -> int:
        return len(self.n_massive)

    @property
    def n_total(self) -> int:
        return int(self.body_offset[-1])

    def sizes(self) -> np.ndarray:
        return np.diff(self.body_offset)

    def pairs_per_step(self) -> int:
        """Kick pairs per step, both half kicks: 2 * sum(Nm (Nm - 1) + Nt Nm)."""
        n = self.sizes().astype(np.int64)
        nm = self.n_massive.astype(np.int64)
        return int(2 * np.sum(nm * (nm - 1) + (n - nm) * nm))

    def element_rows(self) -> np.ndarray:
        return self.elements.reshape(6, -1)

    def subset(self, systems) -> "Systems":
        """The listed systems as a new batch."""
        idx = np.asarray(systems, dtype=np.int64)
        rows = self.element_rows()
        offs = [0]
        mass, el, nm = [], [], []
        for s in idx:
            b0, b1 = int(self.body_offset[s]), int(self.body_offset[s + 1])
            mass.append(self.mass[b0:b1])
            el.append(rows[:, b0:b1])
            nm.append(int(self.n_massive[s]))
            offs.append(offs[-1] + b1 - b0)
        return Systems(np.array(offs, np.int64), np.array(nm, np.int32), np.concatenate(mass),
                       np.concatenate(el, axis=1).reshape(-1).copy(), self.dt, self.hill_factor, self.steps,
                       None, self.label + "[subset]")


def concat(batches) -> "Systems":
    """Several batches as one (systems in order)."""
    blocks = []
    for b in batches:
        rows = b.element_rows()
        for s in range(b.n_systems):
            b0, b1 = int(b.body_offset[s]), int(b.body_offset[s + 1])
            blocks.append((b.mass[b0:b1], rows[:, b0:b1], int(b.n_massive[s])))
    first = batches[0]
    return _pack(blocks, first.dt, first.hill_factor, first.steps, " + ".join(b.label for b in batches))


def shard(sysm: "Systems", rank: int, world: int) -> "Systems":
    """Contiguous share of the systems for one of `world` replicas."""
    idx = np.array_split(np.arange(sysm.n_systems), world)[rank]
    return sysm.subset(idx)


def _uangle(rng, n):
    return rng.uniform(0.0, TWO_PI, n)


def _pack(blocks, dt, hill, steps, label, names=None) -> Systems:
    """blocks: list of (mass[n], elements[6, n], n_massive) per system."""
    offs = [0]
    masses, els, nms = [], [], []
    for m, e, nm in blocks:
        masses.append(np.asarray(m, np.float64))
        els.append(np.asarray(e, np.float64))
        nms.append(nm)
        offs.append(offs[-1] + len(m))
    return Systems(np.array(offs, np.int64), np.array(nms, np.int32), np.concatenate(masses),
                   np.concatenate(els, axis=1).reshape(-1).copy(), dt, hill, steps, names, label)


def _giants(rng, which=(0, 1, 2, 3)):
    m = np.array([GIANTS[k][0] for k in which])
    a = np.array([GIANTS[k][1] for k in which])
    n = len(which)
    e = rng.uniform(0.0, 0.05, n)
    inc = rng.uniform(0.0, 2.0 * DEG, n)
    return m, np.stack([inc, _uangle(rng, n), _uangle(rng, n), _uangle(rng, n), e, a])


def _test_particles(rng, n, a_lo=150.0, a_hi=1000.0, q_lo=30.0, q_hi=50.0, i_max_deg=30.0):
    a = rng.uniform(a_lo, a_hi, n)
    q = rng.uniform(q_lo, q_hi, n)
    e = 1.0 - q / a
    inc = rng.uniform(0.0, i_max_deg * DEG, n)
    return np.zeros(n), np.stack([inc, _uangle(rng, n), _uangle(rng, n), _uangle(rng, n), e, a])


def outer_solar_system(seed: int = 20261203, n_test: int = 100) -> Systems:
    """Workload 0: Sun + 4 giants + a distant planet (m 1.5e-5, a 500 AU, e 0.25,
    i 20 deg) + 100 massless test particles (a U[150,1000], q U[30,50],
    i U[0,30 deg]); dt 0.5 yr, 1e4 steps, changeover at 3 Hill radii."""
    rng = np.random.default_rng(seed)
    gm, ge = _giants(rng)
    pm = np.array([1.5e-5])
    pe = np.array([[20.0 * DEG], [rng.uniform(0, TWO_PI)], [rng.uniform(0, TWO_PI)], [rng.uniform(0, TWO_PI)],
                   [0.25], [500.0]])
    tm, te = _test_particles(rng, n_test)
    m = np.concatenate([gm, pm, tm])
    e = np.concatenate([ge, pe, te], axis=1)
    return _pack([(m, e, 5)], 0.5, 3.0, 10000, "outer-solar-system: 5 massive + 100 test particles")


def embryo_disk(seed: int = 20261204, n_embryos: int = 2000) -> Systems:
    """Workload 1: Sun + Jupiter/Saturn analogues + 2000 embryos (m U[0.025,0.1]
    M_earth, a in [0.5,1.5] AU with surface density ~ a^-1.5, e and i Rayleigh
    0.01 / 0.005); dt 0.01 yr, 1e4 steps, changeover at 3 Hill radii."""
    rng = np.random.default_rng(seed)
    gm, ge = _giants(rng, (0, 1))
    m = rng.uniform(0.025, 0.1, n_embryos) * M_EARTH
    # surface density ~ a^-1.5 -> dN/da ~ a^-0.5 -> sqrt(a) uniform
    u = rng.uniform(0.0, 1.0, n_embryos)
    a = (np.sqrt(0.5) + u * (np.sqrt(1.5) - np.sqrt(0.5))) ** 2
    e = rng.rayleigh(0.01, n_embryos)
    inc = rng.rayleigh(0.005, n_embryos)
    ee = np.stack([inc, _uangle(rng, n_embryos), _uangle(rng, n_embryos), _uangle(rng, n_embryos), e, a])
    mm = np.concatenate([gm, m])
    el = np.concatenate([ge, ee], axis=1)
    return _pack([(mm, el, len(mm))], 0.01, 3.0, 10000, f"embryo-disk: {len(mm)} massive bodies")


def sweep(seed: int = 20261205, n_systems: int = 4096, nt_lo: int = 64, nt_hi: int = 1024) -> Systems:
    """Workload 2: n_systems independent systems, each Sun + 4 giants + a distant
    planet (m U[5,10] M_earth, a U[300,800], e U[0.1,0.5], i U[0,30 deg]) +
    U{64..1024} test particles with the workload-0 distribution; dt 0.5 yr."""
    rng = np.random.default_rng(seed)
    blocks = []
    for _ in range(n_systems):
        gm, ge = _giants(rng)
        pm = np.array([rng.uniform(5.0, 10.0) * M_EARTH])
        pe = np.array([[rng.uniform(0, 30.0 * DEG)], [rng.uniform(0, TWO_PI)], [rng.uniform(0, TWO_PI)],
                       [rng.uniform(0, TWO_PI)], [rng.uniform(0.1, 0.5)], [rng.uniform(300.0, 800.0)]])
        nt = int(rng.integers(nt_lo, nt_hi + 1))
        tm, te = _test_particles(rng, nt)
        blocks.append((np.concatenate([gm, pm, tm]), np.concatenate([ge, pe, te], axis=1), 5))
    return _pack(blocks, 0.5, 3.0, 10000, f"sweep: {n_systems} systems x (5 massive + U{{{nt_lo}..{nt_hi}}} tp)")


def planetesimal_disk(seed: int = 20261207, n_planetesimals: int = 8192, n_test: int = 131072) -> Systems:
    """Workload 4: Sun + 4 giants + 8192 planetesimals (m log-U[1e-9,1e-7], a
    U[5,40], e/i Rayleigh 0.02/0.01) + 131072 test particles (a U[30,1000],
    q U[25,60], i U[0,40 deg]); dt 0.25 yr, 1e3 steps."""
    rng = np.random.default_rng(seed)
    gm, ge = _giants(rng)
    n = n_planetesimals
    pm = np.exp(rng.uniform(np.log(1e-9), np.log(1e-7), n))
    pe = np.stack([rng.rayleigh(0.01, n), _uangle(rng, n), _uangle(rng, n), _uangle(rng, n), rng.rayleigh(0.02, n),
                   rng.uniform(5.0, 40.0, n)])
    tm, te = _test_particles(rng, n_test, 30.0, 1000.0, 25.0, 60.0, 40.0)
    m = np.concatenate([gm, pm, tm])
    el = np.concatenate([ge, pe, te], axis=1)
    return _pack([(m, el, 4 + n)], 0.25, 3.0, 1000, f"planetesimal-disk: {4 + n} massive + {n_test} tp")


def hard_drifts(seed: int = 20261211, n: int = 3 * 65536, dt: float = 0.1) -> Systems:
    """Kepler drifts the benchmark workloads rarely make, for the learned warm
    start: massless test particles around the Sun alone (every step a pure
    two-body drift), one third each on bound orbits with e U[0,0.99] anywhere
    on the orbit (perihelion q log-U[0.2,5] AU), on bound orbits with e
    U[0.5,0.99] within 1.5 rad of true anomaly from perihelion (q log-U[0.05,1]),
    and on hyperbolic orbits with e U[1.02,4] within 0.9 of the asymptotic true
    anomaly (q log-U[0.05,2]); random orientations; dt 0.1 yr (G = 1: a circular
    orbit at 1 AU takes 2 pi yr).  The state is cartesian (extra["pos"],
    extra["vel"]; there is no massive body, so democratic-heliocentric equals
    heliocentric velocity); `elements` is left empty."""
    rng = np.random.default_rng(seed)
    k = n // 3
    parts = []
    for cls, m in (("any", k), ("peri", k), ("hyp", n - 2 * k)):
        if cls == "any":
            e = rng.uniform(0.0, 0.99, m)
            q = np.exp(rng.uniform(np.log(0.2), np.log(5.0), m))
            f = rng.uniform(-np.pi, np.pi, m)
        elif cls == "peri":
            e = rng.uniform(0.5, 0.99, m)
            q = np.exp(rng.uniform(np.log(0.05), np.log(1.0), m))
            f = rng.uniform(-1.5, 1.5, m)
        else:
            e = rng.uniform(1.02, 4.0, m)
            q = np.exp(rng.uniform(np.log(0.05), np.log(2.0), m))
            f = rng.uniform(-0.9, 0.9, m) * np.arccos(-1.0 / e)
        p = q * (1.0 + e)
        r = p / (1.0 + e * np.cos(f))
        x = np.stack([r * np.cos(f), r * np.sin(f), np.zeros(m)])
        v = np.stack([-np.sin(f), e + np.cos(f), np.zeros(m)]) / np.sqrt(p)
        inc = np.arccos(rng.uniform(-1.0, 1.0, m))
        node, peri = _uangle(rng, m), _uangle(rng, m)
        cw, sw, co, so, ci, si = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
        rot = np.array([[co * cw - so * sw * ci, -co * sw - so * cw * ci],
                        [so * cw + co * sw * ci, -so * sw + co * cw * ci],
                        [sw * si, cw * si]])  # columns: perihelion direction, its normal in the plane
        parts.append((np.einsum("ijm,jm->im", rot, x[:2]), np.einsum("ijm,jm->im", rot, v[:2])))
    pos = np.concatenate([a for a, _ in parts], axis=1)
    vel = np.concatenate([b for _, b in parts], axis=1)
    out = Systems(np.array([0, n], np.int64), np.array([0], np.int32), np.zeros(n), np.zeros(0), dt, 3.0, 100,
                  None, f"hard drifts: {n} test particles (e up to 0.99 near perihelion, hyperbolic), dt {dt}")
    out.extra["pos"] = pos.reshape(-1).copy()
    out.extra["vel"] = vel.reshape(-1).copy()
    return out


WORKLOADS = {0: outer_solar_system, 1: embryo_disk, 2: sweep, 4: planetesimal_disk}


# ---------------------------------------------------------------------------
# JSON system config (reference src/simutils.cuh:232-301)
# ---------------------------------------------------------------------------
def to_json(sysm: Systems, path: str, system: int = 0, sweeps: Optional[List[dict]] = None, **options) -> None:
    """Write one system in the reference's config schema (bodies[] with name,
    mass and the six elements; optional sweeps[]) plus optional run keys."""
    b0, b1 = int(sysm.body_offset[system]), int(sysm.body_offset[system + 1])
    rows = sysm.element_rows()
    bodies = []
    for j in range(b0, b1):
        d = {"name": sysm.names[j] if sysm.names else f"body-{j - b0}", "mass": float(sysm.mass[j])}
        for k, key in enumerate(ELEMENT_KEYS):
            d[key] = float(rows[k, j])
        bodies.append(d)
    doc = {"bodies": bodies}
    if sweeps is not None:
        doc["sweeps"] = sweeps
    doc.update(options)
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


def from_json(path: str) -> dict:
    """Read a config; returns {"mass", "elements" (6 x n), "names", "sweeps", "options"}."""
    with open(path) as f:
        doc = json.load(f)
    bodies = doc["bodies"]
    n = len(bodies)
    el = np.zeros((6, n))
    mass = np.zeros(n)
    names = []
    for j, b in enumerate(bodies):
        names.append(b.get("name", ""))
        mass[j] = b["mass"]
        for k, key in enumerate(ELEMENT_KEYS):
            el[k, j] = b[key]
    opts = {k: v for k, v in doc.items() if k not in ("bodies", "sweeps")}
    return {"mass": mass, "elements": el, "names": names, "sweeps": doc.get("sweeps", []), "options": opts}


def count_massive(mass) -> int:
    """Number of bodies heavier than 1e-12 (src/mercurius.cu:4-15)."""
    return int(np.sum(np.asarray(mass) > MASSIVE_THRESHOLD))


def p9_sweep(seed: int = 20261209, n_sweeps: int = 32) -> Systems:
    """The reference's own workload: the Planet Nine configuration of
    p9_config.py (Planet Nine + 4 giants + 10235 TNOs) as n_sweeps systems,
    system k taking sweep k's elements for body 0 with mean anomaly 0 and the
    body's mass unchanged (as mint does, src/mercurius.cu:133-164); the
    reference's dt 0.8219 yr and changeover at 1 Hill radius."""
    import p9_config

    doc = p9_config.p9_config(seed, n_sweeps)
    bodies = doc["bodies"]
    n = len(bodies)
    mass = np.array([b["mass"] for b in bodies])
    base = np.array([[b[k] for b in bodies] for k in ELEMENT_KEYS])
    nm = int(np.sum(mass > MASSIVE_THRESHOLD))
    blocks = []
    for sw in doc["sweeps"]:
        el = base.copy()
        el[:, 0] = [sw[k] for k in ELEMENT_KEYS]
        el[3, 0] = 0.0
        blocks.append((mass, el, nm))
    return _pack(blocks, 0.8219, 1.0, 1000, f"p9 sweep: {n_sweeps} systems x {n} bodies ({nm} massive)",
                 names=None)
