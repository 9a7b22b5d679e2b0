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


def test_bc_reflecting_device_matches_reference(wx, golden_drivers):
    """Rie_prob_2d_rs.apply_bc_reflecting on a random square array (every ghost starts as
    noise): the device fill equals the reference's output bit for bit."""
    import torch
    from weno_ext import problems
    a = torch.from_numpy(golden_drivers["bc/rand_sq"].copy()).cuda()
    got = problems.bc_reflecting_device(a).cpu().numpy()
    assert np.array_equal(got, golden_drivers["bc/reflecting"])


def test_bc_reflecting_device_strided_view(wx, golden_drivers):
    """The fill through a strided (transposed) view writes the same cells."""
    import torch
    from weno_ext import problems
    a = torch.from_numpy(golden_drivers["bc/rand_sq"].transpose(1, 0, 2).copy()).cuda().permute(1, 0, 2)
    problems.bc_reflecting_device(a)
    assert np.array_equal(a.cpu().numpy(), golden_drivers["bc/reflecting"])


def test_bc_reflecting_rejects_non_square(wx):
    import torch
    from weno_ext import problems
    with pytest.raises(ValueError):
        problems.bc_reflecting_device(torch.zeros((20, 17, 8), dtype=torch.float64, device="cuda"))


def test_reference_quadrant_device(wx, golden_drivers):
    """Rie_prob_2d_rs.init (reference states, split at 0.75 nx, reflecting fill) on the
    device equals the driver's own array (drivers.npz rie/q0, 16 x 16)."""
    from weno_ext import problems
    got = problems.reference_quadrant_device(16).cpu().numpy()
    assert np.array_equal(got, golden_drivers["rie/q0"])


def test_refac_device(wx, golden_drivers):
    """unitest.init_refac on the device equals the driver's own array and bound
    (drivers.npz dmr/q0, 40 x 10 on [0,4]x[0,1])."""
    from weno_ext import problems
    q, bound = problems.refac_device(40, 10, 4.0, 1.0)
    assert bound == int(golden_drivers["dmr/bound"])
    assert np.array_equal(q.cpu().numpy(), golden_drivers["dmr/q0"])


def test_refac_device_drives_the_dmr_replay(wx, orc, golden_drivers):
    """The device set-up feeds the solver's oblique-shock loop: 4 exact steps from it equal
    the oracle's double_mach_reflection loop from the driver's own array."""
    from weno_ext import problems
    q, bound = problems.refac_device(40, 10, 4.0, 1.0)
    s = wx.Solver(40, 10, 0.1, 1.4, mode="exact", cons=True, force_hlle=True, cfl=0.1, bc="dmr", bound=bound)
    s.set_state(q)
    s.run(4)
    ref = golden_drivers["dmr/q0"].copy()
    for _ in range(4):
        dt = 0.1 * 0.1 / orc.cfl_cmax(ref, 40, 10, 1.4)
        orc.rk3_step(ref, 40, 10, 0.1, dt, 1.4, True, (0.2, 1.0), True, bc="dmr", bound=bound)
    assert np.array_equal(s.state(), ref)
