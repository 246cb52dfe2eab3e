"""Float64 numpy restatement of the warm-start network and its gradient.
TEST INFRASTRUCTURE: the checker of the GPU training kernels (gradient check)
and of the GPU inference.

Blob layout (MERC_MLP_BLOB = 1267 floats): W1[32][4], b1[32], W2[32][32],
b2[32], W3[32], b3, in_mean[4], in_scale[4], out_mean, out_scale,
box_lo[4], box_hi[4].  Samples: 5 floats (ln x1, x2, x3, x4, target y); the
guess is s = (dt / r0) exp(z), z = -x1 x3 / (2 (1 + x1^2)) + y x1^2 / (1 + x1^2)
(p9-integrator_gb300/csrc/merc_mlp.cuh).
"""
import numpy as np

H = 32
NET = H * 4 + H + H * H + H + H + 1
BLOB = NET + 18
W1, B1 = 0, H * 4
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
IN_MEAN, IN_SCALE, OUT_MEAN, OUT_SCALE, BOX_LO, BOX_HI = NET, NET + 4, NET + 8, NET + 9, NET + 10, NET + 14


def unpack(blob):
    b = np.asarray(blob, np.float64)
    return (b[W1:B1].reshape(H, 4), b[B1:W2], b[W2:B2].reshape(H, H), b[B2:W3], b[W3:B3], b[B3])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_and_grad(blob, samples):
    """Mean 0.5 (net(xn) - t)^2 over the samples and its gradient (float64)."""
    b = np.asarray(blob, np.float64)
    S = np.asarray(samples, np.float64).reshape(-1, 5)
    w1, b1, w2, b2, w3, b3 = unpack(b)
    xn = (S[:, :4] - b[IN_MEAN:IN_MEAN + 4]) * b[IN_SCALE:IN_SCALE + 4]
    t = (S[:, 4] - b[OUT_MEAN]) * b[OUT_SCALE]
    z1 = xn @ w1.T + b1
    h1 = silu(z1)
    z2 = h1 @ w2.T + b2
    h2 = silu(z2)
    y = h2 @ w3 + b3
    e = y - t
    n = S.shape[0]
    d2 = (e[:, None] * w3[None, :]) * dsilu(z2)
    d1 = (d2 @ w2) * dsilu(z1)
    g = np.zeros(NET)
    g[W1:B1] = (d1.T @ xn).reshape(-1) / n
    g[B1:W2] = d1.sum(0) / n
    g[W2:B2] = (d2.T @ h1).reshape(-1) / n
    g[B2:W3] = d2.sum(0) / n
    g[W3:B3] = (e[:, None] * h2).sum(0) / n
    g[B3] = e.sum() / n
    return float(0.5 * np.mean(e * e)), g


def guess(blob, pos, vel, dt):
    """Warm-start guess of the universal anomaly for drift inputs (3 x n); NaN
    where the network is not consulted (outside its box, or x1 < 0.03)."""
    b = np.asarray(blob, np.float64)
    x = np.asarray(pos).reshape(3, -1)
    v = np.asarray(vel).reshape(3, -1)
    r0 = np.sqrt((x * x).sum(0))
    eta = (x * v).sum(0)
    v2 = (v * v).sum(0)
    s0 = dt / r0
    f = np.stack([dt / r0 ** 1.5, r0 * v2, eta / np.sqrt(r0), np.where(2 - r0 * v2 < 0, 1.0, -1.0)], 1)
    f = f.astype(np.float32).astype(np.float64)
    u = f.copy()
    u[:, 0] = np.log(f[:, 0])
    inside = np.all((u >= b[BOX_LO:BOX_LO + 4]) & (u <= b[BOX_HI:BOX_HI + 4]), axis=1) & (f[:, 0] >= np.float32(0.03))
    w1, b1, w2, b2, w3, b3 = unpack(b)
    xn = (u - b[IN_MEAN:IN_MEAN + 4]) * b[IN_SCALE:IN_SCALE + 4]
    yn = silu(silu(xn @ w1.T + b1) @ w2.T + b2) @ w3 + b3
    y = yn / b[OUT_SCALE] + b[OUT_MEAN]
    q = f[:, 0] ** 2
    z = (y * q - 0.5 * f[:, 0] * f[:, 2]) / (1 + q)
    return np.where(inside, s0 * np.exp(z), np.nan)
