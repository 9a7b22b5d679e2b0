"""Out-of-range and unwritten-data detection without a sanitizer: every
workspace byte and every output element starts as a NaN bit pattern (0xFF..),
so a kernel that reads scratch it did not write, or leaves an output element
unwritten, turns the bit-exact comparison with the oracle red."""

import numpy as np
import pytest

from states import noisy, quadrant

pytestmark = pytest.mark.gpu
G = 1.4


def _nan_bytes(torch, nbytes):
    return torch.full((max(nbytes, 1),), 0xFF, dtype=torch.uint8, device="cuda")


def _nan_out(torch, shape):
    return _nan_bytes(torch, int(np.prod(shape)) * 8).view(torch.float64)[: int(np.prod(shape))].view(*shape)


@pytest.mark.parametrize("shape", [(23, 31), (40, 17)])
@pytest.mark.parametrize("cons,hlle", [(False, True), (True, False), (False, False), (True, True)])
def test_l_local_with_nan_scratch(wx, orc, shape, cons, hlle):
    import torch
    from weno_ext import _lib
    L = _lib.load()
    q = noisy(np.random.default_rng(41), *shape)
    u = torch.from_numpy(q).cuda()
    m, n, c = q.shape
    s = u.stride()
    out = _nan_out(torch, (m - 6, n - 6, 4))
    wsb = L.weno_l_local_workspace(m, n, int(hlle))
    ws = _nan_bytes(torch, wsb)
    _lib.check(L.weno_l_local(u.data_ptr(), m, n, c, s[0], s[1], s[2], 0.01, G, int(hlle), 0.05, 0.4, int(cons),
                              _lib.EXACT, out.data_ptr(), ws.data_ptr(), wsb, None), "l_local")
    torch.cuda.synchronize()
    ref = orc.l_local_py(q, 0.01, G, hlle, (0.05, 0.4), cons)
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("ydir", [0, 1])
@pytest.mark.parametrize("cons", [False, True])
def test_reconstruct_and_riemann_with_nan_scratch(wx, orc, ydir, cons):
    import torch
    from weno_ext import _lib
    L = _lib.load()
    q = quadrant(np.random.default_rng(42), 19, 26)
    u = torch.from_numpy(q).cuda()
    m, n, c = q.shape
    s = u.stride()
    shp = (m - 6, n - 5, 4) if ydir else (m - 5, n - 6, 4)
    outs = [_nan_out(torch, shp) for _ in range(4)]
    wsb = L.weno_reconstruct_workspace(m, n, ydir)
    ws = _nan_bytes(torch, wsb)
    _lib.check(L.weno_reconstruct(u.data_ptr(), m, n, c, s[0], s[1], s[2], G, ydir, int(cons), _lib.EXACT,
                                  *[o.data_ptr() for o in outs], ws.data_ptr(), wsb, None), "reconstruct")
    torch.cuda.synchronize()
    refs = (orc.weno_y_py if ydir else orc.weno_x_py)(q, G, cons=cons)
    for got, ref in zip(outs, refs):
        assert np.array_equal(got.cpu().numpy(), ref)
    # the blend Riemann solver on those faces (HLLC, HLLE, sensor) with NaN scratch
    rm, rn = shp[0], shp[1]
    rout = _nan_out(torch, (rm, rn, 4))
    rwsb = L.weno_riemann_workspace(rm, rn, 2)
    rws = _nan_bytes(torch, rwsb)
    _lib.check(L.weno_riemann(*[o.data_ptr() for o in outs], rm, rn, G, ydir, 2, 0.05, 0.4, _lib.EXACT,
                              rout.data_ptr(), rws.data_ptr(), rwsb, None), "riemann")
    torch.cuda.synchronize()
    fn = orc.hllc_hlle_y_rs_py if ydir else orc.hllc_hlle_x_rs_py
    ref = fn(*refs, G, 0.05, 0.4, False)
    assert np.array_equal(rout.cpu().numpy(), ref)


def test_solver_and_batch_with_nan_filled_buffers(wx, orc, golden_drivers, monkeypatch):
    """With WENO_DEBUG_NAN_FILL=1 the solver's state, stage and workspace buffers and
    the batch pools start as NaN bit patterns: the exact runs still equal the oracle's
    and the reference drivers' own runs bit for bit."""
    monkeypatch.setenv("WENO_DEBUG_NAN_FILL", "1")
    rng = np.random.default_rng(43)
    n = 20
    q0 = orc.bc_reflecting(quadrant(rng, n, n))
    ref = q0.copy()
    for _ in range(4):
        dt = 0.45 * (1.0 / n) / orc.cfl_cmax(ref, n, n, G)
        orc.rk3_step(ref, n, n, 1.0 / n, dt, G, False, (0.05, 0.4), False)
    s = wx.Solver(n, n, 1.0 / n, G, mode="exact", cons=False, force_hlle=False, jp_cri=(0.05, 0.4), cfl=0.45)
    s.set_state(q0)
    s.run(4)
    assert np.array_equal(s.state(), ref)
    g = golden_drivers
    d = wx.Solver(40, 10, 0.1, G, cons=True, force_hlle=True, jp_cri=(10000, 11000), cfl=0.1, bc="dmr",
                  bound=int(g["dmr/bound"]))
    d.set_state(g["dmr/q0"])
    d.run(4, t_final=0.01)
    assert np.array_equal(d.state(), g["dmr/q_final"])
    # batch: two uneven solves, exact FP64, against the oracle's runs
    qa = orc.sync_primitives(orc.bc_transmissive(quadrant(rng, 37, 21)), G)
    qb = orc.sync_primitives(orc.bc_transmissive(quadrant(rng, 18, 45)), G)
    b = wx.Batch(wx.Batch.pool_cells([(37, 21), (18, 45)], 64), 2, precision=64, mode="exact", cons=False,
                 force_hlle=True, jp_cri=(0.2, 1.0), cfl=0.45)
    sa = b.add(qa, 1.0 / 37, max_steps=3)
    sb = b.add(qb, 1.0 / 45, max_steps=3)
    b.run(3)
    for slot, q, nx, ny in ((sa, qa, 37, 21), (sb, qb, 18, 45)):
        r = q.copy()
        for _ in range(3):
            dt = 0.45 * (1.0 / max(nx, ny)) / orc.cfl_cmax(r, nx, ny, G)
            orc.rk3_step(r, nx, ny, 1.0 / max(nx, ny), dt, G, True, (0.2, 1.0), False)
        assert np.array_equal(b.state(slot)[3:-3, 3:-3, :4], r[3:-3, 3:-3, :4])
