"""Seeded synthetic states shared by the tests and the benchmark harness."""

import numpy as np


def quadrant(rng, nx, ny, split=0.5, gamma=1.4, channels=8, prim=True):
    """Four-quadrant Riemann state: per quadrant rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]."""
    q = np.zeros((nx + 6, ny + 6, channels))
    si = 3 + int(split * nx)
    sj = 3 + int(split * ny)
    for a, b in ((slice(None, si), slice(None, sj)), (slice(si, None), slice(None, sj)),
                 (slice(None, si), slice(sj, None)), (slice(si, None), slice(sj, None))):
        rho, p = rng.uniform(0.1, 2.0, 2)
        u, v = rng.uniform(-1.0, 1.0, 2)
        q[a, b, 0] = rho
        q[a, b, 1] = rho * u
        q[a, b, 2] = rho * v
        q[a, b, 3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
        if prim and channels >= 8:
            q[a, b, 4], q[a, b, 5], q[a, b, 6], q[a, b, 7] = rho, u, v, p
    return q


def smooth(rng, m, n, channels=8, gamma=1.4, amp=0.3):
    x = np.linspace(0, 1, m)[:, None]
    y = np.linspace(0, 1, n)[None, :]
    k = rng.uniform(1, 4, 4)
    rho = 1.0 + amp * np.sin(2 * np.pi * k[0] * x + 1.3 * y)
    u = 0.5 * np.cos(2 * np.pi * k[1] * y + x)
    v = 0.4 * np.sin(2 * np.pi * k[2] * (x + y))
    p = 1.0 + 0.2 * np.cos(2 * np.pi * k[3] * x * y)
    q = np.zeros((m, n, channels))
    q[:, :, 0] = rho
    q[:, :, 1] = rho * u
    q[:, :, 2] = rho * v
    q[:, :, 3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return q


def noisy(rng, m, n, channels=8, gamma=1.4):
    """Cell-wise random states (every face a discontinuity), including near-vacuum cells."""
    rho = rng.uniform(0.05, 3.0, (m, n))
    u = rng.uniform(-2, 2, (m, n))
    v = rng.uniform(-2, 2, (m, n))
    p = rng.uniform(0.05, 3.0, (m, n))
    q = np.zeros((m, n, channels))
    q[:, :, 0] = rho
    q[:, :, 1] = rho * u
    q[:, :, 2] = rho * v
    q[:, :, 3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return q


def rel_l1(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).sum()
    return float(np.abs(a - b).sum() / den) if den else float(np.abs(a - b).sum())
