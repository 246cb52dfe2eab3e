"""Two-body positions and velocities in closed form (mu = 1), for known-answer
tests of the drift: with no massive bodies the Mercurius step is a pure
Kepler drift, so after time t every body is on its initial ellipse at mean
anomaly M0 + t a^-3/2."""
import numpy as np


def kepler_E(M, e):
    """Eccentric anomaly of E - e sin E = M (e < 1), Newton to convergence."""
    M = np.mod(M, 2 * np.pi)
    E = np.where(e < 0.8, M, np.pi * np.ones_like(M))
    for _ in range(60):
        f = E - e * np.sin(E) - M
        d = f / (1.0 - e * np.cos(E))
        E = E - d
        if np.all(np.abs(d) <= 1e-17 * np.maximum(1.0, np.abs(E))):
            break
    return E


def state(elements, t):
    """elements: 6 x n rows (inclination, node, argument of perihelion, mean
    anomaly, e, a); returns pos, vel (3 x n) at time t."""
    inc, node, peri, M0, e, a = elements
    n = a ** -1.5
    E = kepler_E(M0 + n * t, e)
    cE, sE = np.cos(E), np.sin(E)
    ci, si, co, so, ca, sa = np.cos(inc), np.sin(inc), np.cos(node), np.sin(node), np.cos(peri), np.sin(peri)
    P = np.stack([ca * co - sa * so * ci, ca * so + sa * co * ci, sa * si])
    Q = np.stack([-sa * co - ca * so * ci, -sa * so + ca * co * ci, ca * si])
    b = np.sqrt(1.0 - e * e)
    x, y = a * (cE - e), a * b * sE
    q = np.sqrt(1.0 / a) / (1.0 - e * cE)
    vx, vy = -sE * q, b * cE * q
    return P * x + Q * y, P * vx + Q * vy


def test_particle_batch(seed=11):
    """Two systems of massless bodies only: 40 and 25 bodies, a U[1, 5] AU,
    e U[0, 0.5], i U[0, 30 deg], angles uniform."""
    rng = np.random.default_rng(seed)
    sizes = [40, 25]
    n = sum(sizes)
    el = np.stack([rng.uniform(0, np.pi / 6, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n),
                   rng.uniform(0, 2 * np.pi, n), rng.uniform(0.0, 0.5, n), rng.uniform(1.0, 5.0, n)])
    off = np.array([0, sizes[0], n], np.int64)
    nm = np.zeros(2, np.int32)
    return off, nm, np.zeros(n), el
