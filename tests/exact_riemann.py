"""Exact solution of the 1-D Euler Riemann problem (ideal gas), test helper.

The classical two-rarefaction / two-shock pressure function with a Newton
iteration for the star pressure, then sampling of the self-similar solution
(E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid Dynamics",
3rd ed., chapter 4).  Used to check the solver on the Sod shock tube.
"""

from __future__ import annotations

import math

import numpy as np


def _f(p, rho, pk, ck, g):
    """Pressure function f_K and its derivative for one side."""
    if p > pk:  # shock
        a = 2.0 / ((g + 1.0) * rho)
        b = (g - 1.0) / (g + 1.0) * pk
        s = math.sqrt(a / (p + b))
        return (p - pk) * s, s * (1.0 - 0.5 * (p - pk) / (p + b))
    # rarefaction
    r = p / pk
    return 2.0 * ck / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0), \
        1.0 / (rho * ck) * r ** (-(g + 1.0) / (2.0 * g))


def star_state(left, right, g=1.4, tol=1e-14):
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    p = max(tol, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dl = _f(p, rl, pl, cl, g)
        fr, dr = _f(p, rr, pr, cr, g)
        dp = (fl + fr + ur - ul) / (dl + dr)
        pn = max(tol, p - dp)
        if abs(pn - p) <= tol * 0.5 * (pn + p):
            p = pn
            break
        p = pn
    fl, _ = _f(p, rl, pl, cl, g)
    fr, _ = _f(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(left, right, s, g=1.4):
    """(rho, u, p) at the similarity coordinate s = (x - x0) / t (array)."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    ps, us = star_state(left, right, g)
    s = np.asarray(s, dtype=np.float64)
    rho, u, p = np.empty_like(s), np.empty_like(s), np.empty_like(s)
    gm = (g - 1.0) / (g + 1.0)
    for idx, x in np.ndenumerate(s):
        if x <= us:  # left of the contact
            if ps > pl:  # left shock
                sl = ul - cl * math.sqrt((g + 1.0) / (2.0 * g) * ps / pl + (g - 1.0) / (2.0 * g))
                if x <= sl:
                    v = (rl, ul, pl)
                else:
                    v = (rl * (ps / pl + gm) / (gm * ps / pl + 1.0), us, ps)
            else:  # left rarefaction
                csl = cl * (ps / pl) ** ((g - 1.0) / (2.0 * g))
                if x <= ul - cl:
                    v = (rl, ul, pl)
                elif x >= us - csl:
                    v = (rl * (ps / pl) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) * (cl + (g - 1.0) / 2.0 * (ul - x))
                    uu = 2.0 / (g + 1.0) * (cl + (g - 1.0) / 2.0 * ul + x)
                    v = (rl * (c / cl) ** (2.0 / (g - 1.0)), uu, pl * (c / cl) ** (2.0 * g / (g - 1.0)))
        else:  # right of the contact
            if ps > pr:  # right shock
                sr = ur + cr * math.sqrt((g + 1.0) / (2.0 * g) * ps / pr + (g - 1.0) / (2.0 * g))
                if x >= sr:
                    v = (rr, ur, pr)
                else:
                    v = (rr * (ps / pr + gm) / (gm * ps / pr + 1.0), us, ps)
            else:  # right rarefaction
                csr = cr * (ps / pr) ** ((g - 1.0) / (2.0 * g))
                if x >= ur + cr:
                    v = (rr, ur, pr)
                elif x <= us + csr:
                    v = (rr * (ps / pr) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) * (cr - (g - 1.0) / 2.0 * (ur - x))
                    uu = 2.0 / (g + 1.0) * (-cr + (g - 1.0) / 2.0 * ur + x)
                    v = (rr * (c / cr) ** (2.0 / (g - 1.0)), uu, pr * (c / cr) ** (2.0 * g / (g - 1.0)))
        rho[idx], u[idx], p[idx] = v
    return rho, u, p


SOD_LEFT = (1.0, 0.0, 1.0)
SOD_RIGHT = (0.125, 0.0, 0.1)


def sod_strip(nx, ny=3, gamma=1.4, x0=0.5):
    """The drivers' (nx+6, ny+6, 8) array of the Sod tube along x on [0, 1]."""
    q = np.zeros((nx + 6, ny + 6, 8))
    xc = (np.arange(nx + 6) - 3 + 0.5) / nx
    left = xc < x0
    for mask, (r, u, p) in ((left, SOD_LEFT), (~left, SOD_RIGHT)):
        q[mask, :, 4], q[mask, :, 5], q[mask, :, 6], q[mask, :, 7] = r, u, 0.0, p
    q[..., 0] = q[..., 4]
    q[..., 1] = q[..., 4] * q[..., 5]
    q[..., 2] = 0.0
    q[..., 3] = q[..., 7] / (gamma - 1.0) + 0.5 * q[..., 4] * q[..., 5] ** 2
    return q
