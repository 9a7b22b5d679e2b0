"""Device generators of the initial data equal the numpy generators bit for bit."""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx,ny,seed", [(10, 12, 3), (64, 33, 7), (301, 128, 11)])
def test_quadrant_device(wx, nx, ny, seed):
    from weno_ext import problems
    got = problems.quadrant_device(nx, ny, seed=seed).cpu().numpy()
    assert np.array_equal(got, problems.quadrant(nx, ny, seed=seed))


@pytest.mark.parametrize("nx,ny,lx,ly,mach,deg", [(40, 10, 4.0, 1.0, 10.0, 60.0), (96, 64, 1.5, 1.0, 3.3, 41.0),
                                                  (200, 50, 4.0, 1.0, 7.7, 72.5)])
def test_oblique_shock_device(wx, nx, ny, lx, ly, mach, deg):
    from weno_ext import problems
    th = math.radians(deg)
    q, b, post = problems.oblique_shock(nx, ny, lx, ly, mach, th)
    qd, bd, postd = problems.oblique_shock_device(nx, ny, lx, ly, mach, th)
    assert bd == b
    assert np.array_equal(postd, post)
    assert np.array_equal(qd.cpu().numpy(), q)
