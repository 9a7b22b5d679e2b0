"""The device-resident SSP-RK3 solver against the oracle's restatement of the
drivers and against the golden runs of the reference drivers themselves."""

import numpy as np
import pytest

from states import quadrant, rel_l1

pytestmark = pytest.mark.gpu
G = 1.4


def oracle_run(orc, q, nx, ny, dx, cfl, nstep, t_final=None, bc="transmissive", bound=0, jp=(0.2, 1.0),
               cons=False, hlle=True):
    T, step = 0.0, 0
    while step < nstep and (t_final is None or T < t_final - 1e-12):
        dt = cfl * dx / orc.cfl_cmax(q, nx, ny, G)
        if t_final is not None:
            dt = min(dt, t_final - T)
        orc.rk3_step(q, nx, ny, dx, dt, G, hlle, jp, cons, bc=bc, bound=bound)
        T += dt
        step += 1
    return q, T, step


def rie_init(orc, rng, n):
    q = quadrant(rng, n, n)
    return orc.bc_reflecting(q)


@pytest.mark.parametrize("cons,hlle", [(False, True), (True, False), (False, False), (True, True)])
def test_transmissive_steps_bit_exact(wx, orc, cons, hlle):
    rng = np.random.default_rng(11)
    n = 20
    q0 = rie_init(orc, rng, n)
    ref, T, steps = oracle_run(orc, q0.copy(), n, n, 1 / n, 0.45, 4, jp=(0.05, 0.4), cons=cons, hlle=hlle)
    s = wx.Solver(n, n, 1 / n, G, mode="exact", cons=cons, force_hlle=hlle, jp_cri=(0.05, 0.4), cfl=0.45)
    s.set_state(q0)
    s.run(4)
    got = s.state()
    t, k, st = s.info()
    assert (st & 1) == 0 and k == 4 and t == T
    assert np.array_equal(got, ref), f"max diff {np.abs(got - ref).max()}"


def test_fast_and_fp32_tolerances(wx, orc):
    rng = np.random.default_rng(12)
    n = 24
    q0 = rie_init(orc, rng, n)
    ref, _, _ = oracle_run(orc, q0.copy(), n, n, 1 / n, 0.45, 6)
    fast = wx.Solver(n, n, 1 / n, G, mode="fast", cfl=0.45)
    fast.set_state(q0)
    fast.run(6)
    got = fast.state()
    for k in range(4):
        assert rel_l1(got[3:-3, 3:-3, k], ref[3:-3, 3:-3, k]) <= 1e-10
    f32 = wx.Solver(n, n, 1 / n, G, precision=32, cfl=0.45)
    f32.set_state(q0)
    f32.run(6)
    got = f32.state()
    assert rel_l1(got[3:-3, 3:-3, 0], ref[3:-3, 3:-3, 0]) <= 1e-5


def test_t_final_and_graph(wx, orc):
    rng = np.random.default_rng(13)
    n = 16
    q0 = rie_init(orc, rng, n)
    ref, T, steps = oracle_run(orc, q0.copy(), n, n, 1 / n, 0.5, 100, t_final=0.05)
    for graph in (True, False):
        s = wx.Solver(n, n, 1 / n, G, cfl=0.5)
        s.set_state(q0)
        s.run(steps + 5, t_final=0.05, graph=graph)  # the extra steps are device-side no-ops
        t, k, _ = s.info()
        assert k == steps and t == T
        assert np.array_equal(s.state(), ref)


def test_reference_driver_runs(wx, golden_drivers):
    """Replays of the unchanged reference drivers' own runs (component-wise + HLLE)."""
    g = golden_drivers
    s = wx.Solver(16, 16, 1 / 16, G, cons=True, force_hlle=True, jp_cri=(0.5, 2), cfl=0.3)
    s.set_state(g["rie/q0"])
    s.run(3)
    assert np.array_equal(s.state(), g["rie/q_nstep3"])
    s.set_state(g["rie/q0"])
    s.run(50, t_final=0.02)
    assert np.array_equal(s.state(), g["rie/q_tfinal"])
    d = wx.Solver(40, 10, 0.1, G, cons=True, force_hlle=True, jp_cri=(10000, 11000), cfl=0.1, bc="dmr",
                  bound=int(g["dmr/bound"]))
    d.set_state(g["dmr/q0"])
    d.run(4, t_final=0.01)
    assert np.array_equal(d.state(), g["dmr/q_final"])


def test_dmr_characteristic_hllc(wx, orc, golden_drivers):
    g = golden_drivers
    q0 = g["dmr/q0"]
    bound = int(g["dmr/bound"])
    ref, T, steps = oracle_run(orc, q0.copy(), 40, 10, 0.1, 0.1, 5, bc="dmr", bound=bound, jp=(10000, 11000),
                               cons=False, hlle=False)
    s = wx.Solver(40, 10, 0.1, G, cons=False, force_hlle=False, jp_cri=(10000, 11000), cfl=0.1, bc="dmr", bound=bound)
    s.set_state(q0)
    s.run(5)
    assert np.array_equal(s.state(), ref)


def test_device_state_roundtrip(wx, orc):
    import torch
    rng = np.random.default_rng(14)
    q0 = rie_init(orc, rng, 12)
    s = wx.Solver(12, 12, 1 / 12, G)
    s.set_state(torch.from_numpy(q0).cuda())
    s.run(2)
    a = s.state(device=True).cpu().numpy()
    b = s.state()
    assert np.array_equal(a, b)


def test_characteristic_blow_up_reproduced(wx, orc):
    """The reference algorithm's own NaN blow-up (char reconstruction, low-density
    quadrant, CFL 0.5) is reproduced bit for bit, NaN positions included, and the
    solver reports it as a numeric status."""
    from test_gpu_batch import synced
    q = synced(orc, quadrant(np.random.default_rng(9), 40, 56))
    ref, T, steps = oracle_run(orc, q.copy(), 40, 56, 1 / 56, 0.5, 4, jp=(1e4, 1.1e4), cons=False, hlle=True)
    assert np.isnan(ref).any()
    s = wx.Solver(40, 56, 1 / 56, G, mode="exact", cons=False, force_hlle=True, jp_cri=(1e4, 1.1e4), cfl=0.5)
    s.set_state(q)
    s.run(4)
    got = s.state()
    assert s.info()[2] != 0
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    fin = ~np.isnan(ref)
    assert np.array_equal(got[fin], ref[fin])


def test_pinned_host_buffers_match_pageable(wx, orc):
    """set_state_host / get_state_host on page-locked host memory (the e2e path of
    the benchmark) give the same bits as on pageable memory."""
    import torch
    from weno_ext import _lib
    L = _lib.load()
    nx, ny = 33, 38
    q0 = orc.bc_transmissive(quadrant(np.random.default_rng(17), nx, ny))
    res = []
    for pinned in (False, True):
        s = wx.Solver(nx, ny, 1 / ny, G, mode="exact", cons=False, force_hlle=True, cfl=0.45)
        if pinned:
            src = torch.from_numpy(q0.copy()).pin_memory()
            dst = torch.full((nx + 6, ny + 6, 8), float("nan"), dtype=torch.float64).pin_memory()
            _lib.check(L.weno_solver_set_state_host(s._h, src.data_ptr(), 8), "set_state_host")
            s.run(3)
            _lib.check(L.weno_solver_get_state_host(s._h, dst.data_ptr()), "get_state_host")
            res.append(dst.numpy().copy())
        else:
            s.set_state(q0)
            s.run(3)
            res.append(s.state())
    assert np.isfinite(res[1]).all()
    assert np.array_equal(res[0], res[1])
