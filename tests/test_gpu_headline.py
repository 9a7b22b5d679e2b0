"""Parity of the benchmark's headline workload at its own size.

The bench times the 4096 x 4096 four-quadrant Riemann problem (seed 20261203),
characteristic WENO5 + 2-point Gauss faces + HLLE, SSP-RK3 at CFL 0.45, in FP64
with the FAST arithmetic.  These tests pin that exact configuration:

* the exact arithmetic is bit-identical to the oracle (the restated Rust core
  and numpy driver step, weno.rs:367-632, riemann.rs:191-349,489-541,
  Rie_prob_2d_rs.py:169-207,311-319) after two full steps;
* the FAST arithmetic stays within 1e-10 relative L1 per conserved variable of
  the exact arithmetic over the 25 steps a default benchmark run makes
  (5 warm-up + 20 timed);
* the same FAST-vs-exact bound for the HLLC/HLLE pressure-sensor blend at 2048^2.
"""

import numpy as np
import pytest

from states import rel_l1

pytestmark = pytest.mark.gpu
G = 1.4
N = 4096
SEED = 20261203
KW = dict(cons=False, force_hlle=True, jp_cri=(0.2, 1.0), cfl=0.45)
TOL = 1e-10  # relative L1 per conserved variable, FAST against exact FP64


def _quadrant(n):
    from weno_ext import problems
    return problems.quadrant(n, n, seed=SEED)


def test_headline_exact_bit_identical_to_oracle_two_steps(wx, orc):
    q0 = _quadrant(N)
    s = wx.Solver(N, N, 1.0 / N, G, mode="exact", **KW)
    s.set_state(q0)
    s.run(2)
    got = s.state()
    assert s.info()[1:] == (2, 0)
    s.close()
    orc.set_threads(0)
    ref = q0
    for _ in range(2):
        dt = 0.45 * (1.0 / N) / orc.cfl_cmax(ref, N, N, G)
        orc.rk3_step(ref, N, N, 1.0 / N, dt, G, True, (0.2, 1.0), False)
    assert np.isfinite(ref).all()
    assert np.array_equal(got, ref)


def _fast_vs_exact(wx, n, steps, checkpoints, kw):
    q0 = _quadrant(n)
    sol = {}
    for mode in ("exact", "fast"):
        s = wx.Solver(n, n, 1.0 / n, G, mode=mode, **kw)
        s.set_state(q0)
        sol[mode] = s
    worst = []
    done = 0
    for c in checkpoints:
        for s in sol.values():
            s.run(c - done)
        done = c
        ex, fa = sol["exact"].state(), sol["fast"].state()
        assert np.isfinite(ex).all() and np.isfinite(fa).all()
        worst.append(max(rel_l1(fa[3:-3, 3:-3, k], ex[3:-3, 3:-3, k]) for k in range(4)))
    for s in sol.values():
        assert s.info()[1:] == (steps, 0)
        s.close()
    return worst


def test_headline_fast_tracks_exact_over_bench_steps(wx):
    worst = _fast_vs_exact(wx, N, 25, (5, 15, 25), KW)
    print("fast vs exact, worst relative L1 after 5/15/25 steps:", worst)
    assert max(worst) <= TOL, worst


@pytest.mark.parametrize("jp_cri", [(0.2, 1.0), (1e4, 1.1e4)], ids=["blend", "hllc"])
def test_char_blend_fast_tracks_exact_2048(wx, jp_cri):
    kw = dict(KW, force_hlle=False, jp_cri=jp_cri)
    worst = _fast_vs_exact(wx, 2048, 25, (5, 15, 25), kw)
    print("char blend", jp_cri, "worst relative L1 after 5/15/25 steps:", worst)
    assert max(worst) <= TOL, worst
