"""Sod shock tube on an nx x 3 strip (the set-up of Rie_prob_1D_rs.py) against
the exact Riemann solution: the oracle's driver step converges to it."""

import numpy as np
import pytest

from exact_riemann import SOD_LEFT, SOD_RIGHT, sample, sod_strip, star_state

G = 1.4
T_END = 0.2


def sod_run(orc, nx, cons=True, hlle=True, jp=(0.2, 1.0), cfl=0.4, transpose=False):
    q = sod_strip(nx)
    mx, my = nx, 3
    if transpose:
        q = np.ascontiguousarray(q.transpose(1, 0, 2)[:, :, [0, 2, 1, 3, 4, 6, 5, 7]])
        mx, my = 3, nx
    orc.bc_transmissive(q)
    dx = 1.0 / nx
    t, n = 0.0, 0
    while t < T_END - 1e-12:
        dt = min(cfl * dx / orc.cfl_cmax(q, mx, my, G), T_END - t)
        orc.rk3_step(q, mx, my, dx, dt, G, hlle, jp, cons)
        t += dt
        n += 1
    return q, t, n


def l1_density(q, nx, transpose=False):
    xc = (np.arange(nx) + 0.5) / nx
    rho, _, _ = sample(SOD_LEFT, SOD_RIGHT, (xc - 0.5) / T_END)
    line = q[3:-3, 3:-3, 0] if not transpose else q[3:-3, 3:-3, 0].T
    return float(np.abs(line - rho[:, None]).mean())


def test_exact_star_state():
    # Toro, table 4.2 test 1: p* = 0.30313, u* = 0.92745
    p, u = star_state(SOD_LEFT, SOD_RIGHT, G)
    assert p == pytest.approx(0.30313, abs=1e-5)
    assert u == pytest.approx(0.92745, abs=1e-5)


@pytest.mark.parametrize("hlle,jp", [(True, (0.2, 1.0)), (False, (1e4, 1.1e4))])
def test_sod_converges_to_exact(orc, hlle, jp):
    e = {}
    for nx in (100, 200):
        q, t, _ = sod_run(orc, nx, cons=True, hlle=hlle, jp=jp)
        assert t == pytest.approx(T_END, abs=1e-12)
        # the strip stays uniform across y exactly
        assert np.array_equal(q[3:-3, 3:-3, :4], np.repeat(q[3:-3, 3:4, :4], 3, axis=1))
        e[nx] = l1_density(q, nx)
    assert e[200] < 3.5e-3
    assert e[100] / e[200] > 1.7  # first order at the discontinuities


def test_sod_y_direction_is_the_transpose(orc):
    qx, _, nx_steps = sod_run(orc, 100)
    qy, _, ny_steps = sod_run(orc, 100, transpose=True)
    assert nx_steps == ny_steps
    back = qy.transpose(1, 0, 2)[:, :, [0, 2, 1, 3, 4, 6, 5, 7]]
    assert np.allclose(back[3:-3, 3:-3, :4], qx[3:-3, 3:-3, :4], rtol=0, atol=1e-13)


def test_sod_characteristic_scheme_breaks_down(orc):
    """The reference's characteristic scheme (left eigenvectors scaled by
    0.5/(rho c), not the inverse of the right ones off rho = 1) does not survive
    the Sod tube: the 0.125 density side drives it non-finite."""
    q, _, _ = sod_run(orc, 100, cons=False)
    assert not np.isfinite(q[3:-3, 3:-3, :4]).all()
