"""The double-float (df64) solver mode against the oracle and the native FP64 path.

df64 carries about 48 significant bits in two floats and runs on the FP32
pipes; it is an extra mode beside IEEE FP64, never a substitute for the exact
path.  Tolerances: relative L1 <= 1e-10 per conserved channel against the
oracle after a few steps (the same bar as the fused-FMA FP64 mode).
"""

import numpy as np
import pytest

from states import quadrant, rel_l1

pytestmark = pytest.mark.gpu
G = 1.4
TOL = 1e-10


def oracle_run(orc, q, nx, ny, dx, cfl, nstep, bc="transmissive", bound=0, jp=(0.2, 1.0), cons=False, hlle=True):
    for _ in range(nstep):
        dt = cfl * dx / orc.cfl_cmax(q, nx, ny, G)
        orc.rk3_step(q, nx, ny, dx, dt, G, hlle, jp, cons, bc=bc, bound=bound)
    return q


@pytest.mark.parametrize("cons,hlle", [(False, True), (True, False), (False, False), (True, True)])
def test_df64_against_oracle(wx, orc, cons, hlle):
    rng = np.random.default_rng(21)
    n = 24
    q0 = orc.bc_reflecting(quadrant(rng, n, n))
    ref = oracle_run(orc, q0.copy(), n, n, 1 / n, 0.45, 6, jp=(0.05, 0.4), cons=cons, hlle=hlle)
    s = wx.Solver(n, n, 1 / n, G, precision="df64", cons=cons, force_hlle=hlle, jp_cri=(0.05, 0.4), cfl=0.45)
    s.set_state(q0)
    s.run(6)
    got = s.state()
    t, k, st = s.info()
    assert (st & 1) == 0 and k == 6
    for c in range(4):
        assert rel_l1(got[3:-3, 3:-3, c], ref[3:-3, 3:-3, c]) <= TOL


def test_df64_dmr_golden(wx, orc, golden_drivers):
    g = golden_drivers
    bound = int(g["dmr/bound"])
    s = wx.Solver(40, 10, 0.1, G, precision="df64", cons=True, force_hlle=True, jp_cri=(10000, 11000), cfl=0.1,
                  bc="dmr", bound=bound)
    e = wx.Solver(40, 10, 0.1, G, cons=True, force_hlle=True, jp_cri=(10000, 11000), cfl=0.1, bc="dmr", bound=bound)
    for x in (s, e):
        x.set_state(g["dmr/q0"])
        x.run(4, t_final=0.01)
    got, ref = s.state(), g["dmr/q_final"]
    assert np.array_equal(e.state(), ref)
    assert s.info()[1] == e.info()[1] and s.info()[0] == pytest.approx(e.info()[0], rel=1e-12)
    for c in range(4):
        assert rel_l1(got[3:-3, 3:-3, c], ref[3:-3, 3:-3, c]) <= TOL


def _steps(wx, q0, n, prec, cons, nsteps):
    s = wx.Solver(n, n, 1 / n, G, precision=prec, mode="fast", cfl=0.45, cons=cons)
    s.set_state(q0)
    first_bad = None
    for k in range(nsteps):
        s.run(1)
        if first_bad is None and s.info()[2]:
            first_bad = k
    return s, first_bad


def test_df64_against_native_fp64_large(wx):
    """512^2, 20 steps, component-wise WENO + HLLE: df64 against native FP64 (fast)."""
    rng = np.random.default_rng(22)
    n = 512
    q0 = quadrant(rng, n, n)
    a, _ = _steps(wx, q0, n, 64, True, 20)
    b, _ = _steps(wx, q0, n, "df64", True, 20)
    ia, ib = a.info(), b.info()
    assert ia[1] == ib[1] == 20 and ia[2] == ib[2] == 0
    assert ib[0] == pytest.approx(ia[0], rel=1e-12)
    sa, sb = a.state(), b.state()
    ta, tb = a.totals(), b.totals()
    for c in range(4):
        assert rel_l1(sb[3:-3, 3:-3, c], sa[3:-3, 3:-3, c]) <= 1e-12
        assert tb[c] == pytest.approx(ta[c], rel=1e-12, abs=1e-12)


def test_df64_characteristic_blow_up_matches(wx):
    """The reference's characteristic scheme goes non-finite on this seed (its left
    eigenvectors are not the inverse of the right ones); df64 fails at the same step."""
    rng = np.random.default_rng(22)
    n = 512
    q0 = quadrant(rng, n, n)
    _, ka = _steps(wx, q0, n, 64, False, 6)
    _, kb = _steps(wx, q0, n, "df64", False, 6)
    assert ka is not None and ka == kb


@pytest.mark.parametrize("rv", [1e-9, 1e-20])
def test_df64_near_vacuum_guard(wx, orc, rv):
    """Densities far below 1e-6 send the faces near them through native FP64
    reconstruction.  One step only: from the second step on the reference
    scheme itself runs away on this state (pressures of -1e26 by step 3),
    which native doubles still hold and df64, with the float exponent range,
    turns into non-finite values."""
    rng = np.random.default_rng(23)
    n = 24
    q0 = quadrant(rng, n, n)
    q0[3:9, 3:9, 0] = rv
    q0[3:9, 3:9, 1:3] = 0.0
    q0[3:9, 3:9, 3] = rv / 0.4
    q0[3:9, 3:9, 4] = rv
    q0[3:9, 3:9, 5:7] = 0.0
    q0[3:9, 3:9, 7] = rv
    q0 = orc.bc_reflecting(q0)
    ref = oracle_run(orc, q0.copy(), n, n, 1 / n, 0.3, 1, cons=True)
    s = wx.Solver(n, n, 1 / n, G, precision="df64", cons=True, force_hlle=True, cfl=0.3)
    s.set_state(q0)
    s.run(1)
    got = s.state()
    assert np.isfinite(got).all()
    for c in range(4):
        assert rel_l1(got[3:-3, 3:-3, c], ref[3:-3, 3:-3, c]) <= 1e-12


def test_df64_precision_codes(wx):
    s = wx.Solver(8, 8, 1 / 8, G, precision=48)
    assert s.precision == 48
    with pytest.raises(Exception, match="precision"):
        wx.Solver(8, 8, 1 / 8, G, precision=40)
