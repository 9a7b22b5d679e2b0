"""Seeded initial data of the benchmark configurations, in the drivers' layout.

Every generator returns the reference drivers' (nx+6, ny+6, 8) float64 array:
conserved channels rho, rho*u, rho*v, E and primitive channels rho, u, v, p,
ghost cells included (Rie_prob_2d_rs.py:213-263, unitest.py:169-205).

* ``quadrant`` -- the four-quadrant Riemann problem with per-quadrant
  rho, p ~ U[0.1, 2] and u, v ~ U[-1, 1] (quadrant split at the middle).
* ``reference_quadrant_device`` -- the reference driver's own four-quadrant
  set-up (Rie_prob_2d_rs.init: fixed states, split at 3 + int(0.75 nx),
  reflecting fill), and ``refac_device`` -- its double-Mach set-up
  (unitest.init_refac), both generated on the device bit for bit.
* ``oblique_shock`` -- a planar shock at angle ``theta`` to the lower wall,
  through (x0, 0), Mach ``mach`` into gas at rest (rho = 1.4, p = 1), post-shock
  state from the normal-shock Rankine-Hugoniot relations; lower wall with the
  inflow segment x < x0, as in double_mach_reflection.py / unitest.init_refac.
  The reference's double-Mach set-up (M = 10, 60 degrees) uses the post-shock
  velocity (4.125, -7.1447) (unitest.py:194-197, 215), which is the normal
  velocity 8.25 along (cos 60, -sin 60); the shock normal of a 60-degree line
  is (sin 60, -cos 60), so this generator returns (7.1447, -4.125) for that
  case -- the replay tests use the reference's own arrays instead.
"""

from __future__ import annotations

import math

import numpy as np

GAMMA = 1.4


def _conserve(q, gamma):
    rho, u, v, p = q[..., 4], q[..., 5], q[..., 6], q[..., 7]
    q[..., 0] = rho
    q[..., 1] = rho * u
    q[..., 2] = rho * v
    q[..., 3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return q


def quadrant_states(seed):
    """The four seeded primitive states (rho, u, v, p) of `quadrant`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(4):
        rho, p = rng.uniform(0.1, 2.0, 2)
        u, v = rng.uniform(-1.0, 1.0, 2)
        out.append((rho, u, v, p))
    return out


def quadrant(nx, ny, seed=0, gamma=GAMMA, split=0.5):
    rng = np.random.default_rng(seed)
    q = np.zeros((nx + 6, ny + 6, 8))
    si = 3 + int(split * nx)
    sj = 3 + int(split * ny)
    for a, b in ((slice(None, si), slice(None, sj)), (slice(si, None), slice(None, sj)),
                 (slice(None, si), slice(sj, None)), (slice(si, None), slice(sj, None))):
        rho, p = rng.uniform(0.1, 2.0, 2)
        u, v = rng.uniform(-1.0, 1.0, 2)
        q[a, b, 4], q[a, b, 5], q[a, b, 6], q[a, b, 7] = rho, u, v, p
    return _conserve(q, gamma)


def rankine_hugoniot(mach, theta, rho1=1.4, p1=1.0, gamma=GAMMA):
    """Post-shock (rho, u, v, p) behind a shock of Mach `mach` moving into gas at
    rest, the shock line at angle `theta` (radians) to the x axis, the gas moving
    along the shock normal (sin theta, -cos theta)."""
    m2 = mach * mach
    rho2 = rho1 * (gamma + 1.0) * m2 / ((gamma - 1.0) * m2 + 2.0)
    p2 = p1 * (2.0 * gamma * m2 - (gamma - 1.0)) / (gamma + 1.0)
    w = mach * math.sqrt(gamma * p1 / rho1)
    un = w * (1.0 - rho1 / rho2)
    return rho2, un * math.sin(theta), -un * math.cos(theta), p2


def oblique_shock(nx, ny, lx, ly, mach, theta, x0=1.0 / 6.0, gamma=GAMMA):
    """(q, bound, post8): the drivers' array, the DMR boundary's `bound` row and
    the 8-channel inflow vector for weno_ext.Solver(bc="dmr") / Batch.add."""
    rho2, u2, v2, p2 = rankine_hugoniot(mach, theta, gamma=gamma)
    q = np.zeros((nx + 6, ny + 6, 8))
    q[..., 4], q[..., 5], q[..., 6], q[..., 7] = 1.4, 0.0, 0.0, 1.0
    x = (np.arange(nx + 6) - 3 + 0.5) / nx * lx
    y = (np.arange(ny + 6) - 3 + 0.5) / ny * ly
    behind = y[None, :] - math.tan(theta) * (x[:, None] - x0) >= 0.0
    q[behind, 4], q[behind, 5], q[behind, 6], q[behind, 7] = rho2, u2, v2, p2
    _conserve(q, gamma)
    post = np.zeros(8)
    post[4:] = (rho2, u2, v2, p2)
    post[0] = rho2
    post[1] = rho2 * u2
    post[2] = rho2 * v2
    post[3] = p2 / (gamma - 1.0) + 0.5 * rho2 * (u2 * u2 + v2 * v2)
    # last padded row whose cell centre lies before the shock foot on the wall
    bound = int(3 + math.floor(x0 / (lx / nx) - 0.5))
    # apply the oblique-shock boundary once (the driver's init does, unitest.py:205)
    for i in range(3):
        q[i, :, :] = post
        q[:, ny + 3 + i, :] = q[:, ny + 2, :]
        q[nx + 3 + i, :, :] = q[nx + 2, :, :]
        q[:bound + 1, i, :] = post
        q[bound + 1:bound + 10, i, :] = q[bound + 1:bound + 10, 3, :]
        q[bound + 10:, i, :] = q[bound + 10:, 5 - i, :]
        q[bound + 10:, i, 2] *= -1
        q[bound + 10:, i, 6] *= -1
    return q, bound, post


def batch_shapes(n, lo, hi, seed, max_aspect=4.0):
    """Seeded (nx, ny) pairs: edges log-uniform in [lo, hi], aspect ratio within max_aspect."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        a = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        b = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        if max(a, b) / min(a, b) <= max_aspect:
            out.append((int(round(a)), int(round(b))))
    return out


def quadrant_device(nx, ny, seed=0, gamma=GAMMA, split=0.5):
    """`quadrant` generated on the current CUDA device (a torch float64 tensor)."""
    import ctypes
    import torch
    from . import _lib
    L = _lib.load()
    out = torch.empty((nx + 6, ny + 6, 8), dtype=torch.float64, device="cuda")
    prim = np.ascontiguousarray(np.array(quadrant_states(seed), dtype=np.float64).reshape(16))
    _lib.check(L.weno_init_quadrant(out.data_ptr(), nx, ny, 3 + int(split * nx), 3 + int(split * ny),
                                    prim.ctypes.data, float(gamma), torch.cuda.current_stream().cuda_stream),
               "init_quadrant")
    return out


def oblique_shock_device(nx, ny, lx, ly, mach, theta, x0=1.0 / 6.0, gamma=GAMMA):
    """`oblique_shock` generated on the current CUDA device: (tensor, bound, post8)."""
    import ctypes
    import torch
    from . import _lib
    L = _lib.load()
    out = torch.empty((nx + 6, ny + 6, 8), dtype=torch.float64, device="cuda")
    bound = ctypes.c_int64()
    post = np.zeros(8)
    _lib.check(L.weno_init_oblique_shock(out.data_ptr(), nx, ny, float(lx), float(ly), float(x0), float(mach),
                                         float(theta), 1.4, 1.0, float(gamma), ctypes.byref(bound), post.ctypes.data,
                                         torch.cuda.current_stream().cuda_stream), "init_oblique_shock")
    return out, bound.value, post


# Rie_prob_2d_rs.py:213-254 -- the reference's quadrant states (rho, u, v, p) in the
# order (i < s, j < s), (i >= s, j < s), (i < s, j >= s), (i >= s, j >= s).
REFERENCE_QUADRANTS = ((0.125, 1.0, 1.0, 0.025), (0.5, 0.0, 1.0, 0.25), (0.5, 1.0, 0.0, 0.25), (1.0, 0.0, 0.0, 1.0))


def bc_reflecting_device(q):
    """Rie_prob_2d_rs.apply_bc_reflecting in place on a square (n, n, 8) float64 CUDA tensor."""
    import torch
    from . import _lib
    L = _lib.load()
    if not (isinstance(q, torch.Tensor) and q.is_cuda and q.dtype == torch.float64 and q.dim() == 3):
        raise TypeError("q: expected a 3-D float64 CUDA tensor")
    s = q.stride()
    _lib.check(L.weno_bc_reflecting(q.data_ptr(), *q.shape, *s, torch.cuda.current_stream().cuda_stream),
               "bc_reflecting")
    return q


def reference_quadrant_device(n, gamma=GAMMA):
    """Rie_prob_2d_rs.init on the current CUDA device: the (n+6, n+6, 8) array of the
    reference's four-quadrant problem (square grids, as its reflecting fill requires)."""
    import torch
    from . import _lib
    L = _lib.load()
    out = torch.empty((n + 6, n + 6, 8), dtype=torch.float64, device="cuda")
    si = 3 + int(n * 0.75)
    prim = np.ascontiguousarray(np.array(REFERENCE_QUADRANTS, dtype=np.float64).reshape(16))
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.weno_init_quadrant(out.data_ptr(), n, n, si, si, prim.ctypes.data, float(gamma), st),
               "init_quadrant")
    return bc_reflecting_device(out)


def refac_device(nx, ny, lx=4.0, ly=1.0, gamma=GAMMA):
    """unitest.init_refac on the current CUDA device: (tensor, bound) for
    Solver(bc="dmr", bound=bound) with the driver's own inflow vector."""
    import ctypes
    import torch
    from . import _lib
    L = _lib.load()
    out = torch.empty((nx + 6, ny + 6, 8), dtype=torch.float64, device="cuda")
    bound = ctypes.c_int64()
    _lib.check(L.weno_init_refac(out.data_ptr(), nx, ny, float(lx), float(ly), float(gamma), ctypes.byref(bound),
                                 torch.cuda.current_stream().cuda_stream), "init_refac")
    return out, bound.value
