"""Sod shock tube on the device solver: bit-identical to the oracle's run in
exact mode (both directions), and every precision close to the exact solution."""

import numpy as np
import pytest

from exact_riemann import sod_strip
from test_oracle_sod import T_END, l1_density, sod_run

pytestmark = pytest.mark.gpu
G = 1.4


def device_run(wx, nx, transpose=False, **kw):
    q = sod_strip(nx)
    mx, my = nx, 3
    if transpose:
        q = np.ascontiguousarray(q.transpose(1, 0, 2)[:, :, [0, 2, 1, 3, 4, 6, 5, 7]])
        mx, my = 3, nx
    s = wx.Solver(mx, my, 1.0 / nx, G, cons=True, force_hlle=True, jp_cri=(0.2, 1.0), cfl=0.4, **kw)
    s.set_state(q)
    s.run(10000, t_final=T_END)
    return s


@pytest.mark.parametrize("transpose", [False, True])
def test_sod_bit_exact_against_oracle(wx, orc, transpose):
    nx = 400
    ref, t, n = sod_run(orc, nx, transpose=transpose)
    s = device_run(wx, nx, transpose=transpose)
    ts, ns, st = s.info()
    assert st == 0 and ns == n and ts == t
    assert np.array_equal(s.state(), ref)
    assert l1_density(ref, nx, transpose) < 2e-3


@pytest.mark.parametrize("precision,mode,tol", [(64, "fast", 1e-12), ("df64", "fast", 1e-12), (32, "fast", 1e-5)])
def test_sod_precisions(wx, orc, precision, mode, tol):
    nx = 400
    ref, _, _ = sod_run(orc, nx)
    s = device_run(wx, nx, precision=precision, mode=mode)
    got = s.state()
    assert s.info()[2] == 0
    e_ref, e_got = l1_density(ref, nx), l1_density(got, nx)
    assert abs(e_got - e_ref) <= tol + 1e-3 * e_ref * (precision == 32)
    assert np.abs(got[3:-3, 3:-3, 0] - ref[3:-3, 3:-3, 0]).mean() <= tol
