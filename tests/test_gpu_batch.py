"""The batched solver (fused tile kernels, packed pool, per-solve dt): bit-identical
to the oracle's driver loop in exact FP64, identical for a solve alone and in a
mix, and within tolerance in FP32 and fast FP64."""

import numpy as np
import pytest

from states import quadrant, rel_l1
from test_gpu_solver import oracle_run

pytestmark = pytest.mark.gpu
G = 1.4


def synced(orc, q):
    """A state whose primitive channels equal con2primi of its conserved channels
    (the batched solver computes the first dt from the conserved channels)."""
    q = orc.bc_transmissive(q)
    return orc.sync_primitives(q, G)


@pytest.mark.parametrize("cons,hlle", [(False, True), (True, False), (False, False), (True, True)])
@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4])
def test_exact_batch_matches_oracle(wx, orc, cons, hlle, cfg):
    rng = np.random.default_rng(100 + cfg)
    shapes = [(21, 13), (9, 40), (33, 33)]
    qs = [synced(orc, quadrant(rng, nx, ny)) for nx, ny in shapes]
    b = wx.Batch(50000, 8, precision=64, mode="exact", cons=cons, force_hlle=hlle, jp_cri=(0.05, 0.4), cfl=0.45,
                 tile_config=cfg)
    slots = [b.add(q, 1.0 / max(q.shape[0] - 6, q.shape[1] - 6), max_steps=4) for q in qs]
    b.run(6)  # two extra steps: solves stop at max_steps
    for slot, q, (nx, ny) in zip(slots, qs, shapes):
        ref, T, steps = oracle_run(orc, q.copy(), nx, ny, 1.0 / max(nx, ny), 0.45, 4, jp=(0.05, 0.4), cons=cons,
                                   hlle=hlle)
        inf = b.info(slot)
        assert inf["steps"] == 4 and inf["t"] == T and not inf["active"]
        got = b.state(slot)
        assert np.array_equal(got, ref), f"slot {slot}: max diff {np.abs(got - ref).max()}"


def test_exact_batch_dmr_boundary(wx, orc, golden_drivers):
    g = golden_drivers
    q0 = orc.sync_primitives(g["dmr/q0"].copy(), G)
    bound = int(g["dmr/bound"])
    ref, T, steps = oracle_run(orc, q0.copy(), 40, 10, 0.1, 0.1, 5, bc="dmr", bound=bound, jp=(10000, 11000),
                               cons=False, hlle=False, t_final=0.02)
    b = wx.Batch(20000, 2, precision=64, mode="exact", cons=False, force_hlle=False, jp_cri=(10000, 11000), cfl=0.1)
    s = b.add(q0, 0.1, t_end=0.02, max_steps=5, bc="dmr", bound=bound)
    b.run(7)
    assert b.info(s)["steps"] == steps
    assert np.array_equal(b.state(s), ref)


@pytest.mark.parametrize("precision,mode", [(32, "fast"), (64, "fast"), (64, "exact")])
def test_alone_equals_in_the_mix(wx, orc, precision, mode):
    rng = np.random.default_rng(7)
    shapes = [(64, 17), (30, 95), (48, 48), (20, 77), (100, 31)]
    qs = [synced(orc, quadrant(rng, nx, ny)) for nx, ny in shapes]
    t_ends = [0.05, 0.08, 0.03, 0.06, 0.04]
    kw = dict(precision=precision, mode=mode, cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4), cfl=0.5)
    mix = wx.Batch(200000, 8, **kw)
    slots = [mix.add(q, 1.0 / max(nx, ny), t_end=te) for q, (nx, ny), te in zip(qs, shapes, t_ends)]
    for _ in range(40):
        mix.run(5)
        if not mix.poll()[0].any():
            break
    for k in (0, 2, 4):
        alone = wx.Batch(200000, 2, **kw)
        s = alone.add(qs[k], 1.0 / max(shapes[k]), t_end=t_ends[k])
        for _ in range(40):
            alone.run(5)
            if not alone.info(s)["active"]:
                break
        assert alone.info(s)["t"] == mix.info(slots[k])["t"]
        assert np.array_equal(alone.state(s), mix.state(slots[k]))


def test_fp32_and_fast_against_oracle(wx, orc):
    rng = np.random.default_rng(9)
    nx, ny = 40, 56
    q = synced(orc, quadrant(rng, nx, ny))
    ref, T, steps = oracle_run(orc, q.copy(), nx, ny, 1.0 / 56, 0.5, 8, jp=(1e4, 1.1e4), cons=True, hlle=False)
    for precision, mode, tol in ((32, "fast", 1e-5), (64, "fast", 1e-10)):
        b = wx.Batch(20000, 1, precision=precision, mode=mode, cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4),
                     cfl=0.5)
        s = b.add(q, 1.0 / 56, max_steps=8)
        b.run(8)
        got = b.state(s)
        for k in range(4):
            assert rel_l1(got[3:-3, 3:-3, k], ref[3:-3, 3:-3, k]) <= tol


@pytest.mark.parametrize("cons,hlle", [(True, False), (False, True), (False, False), (True, True)])
def test_staged_fast_against_oracle(wx, orc, cons, hlle):
    """The staged configuration in FAST FP64 (two faces per thread in pass 2) and FP32,
    uneven solves in one batch: within 1e-10 (FP64) / 1e-5 (FP32, component-wise)
    relative L1 of the oracle after 6 steps."""
    # seed 20: states on which the reference's characteristic scheme stays finite and
    # bounded for 10 steps (on many seeded quadrant states it runs away within a few)
    rng = np.random.default_rng(20)
    shapes = [(40, 56), (33, 17), (64, 64)]
    qs = [synced(orc, quadrant(rng, nx, ny)) for nx, ny in shapes]
    refs = [oracle_run(orc, q.copy(), nx, ny, 1.0 / max(nx, ny), 0.45, 6, jp=(0.05, 0.4), cons=cons, hlle=hlle)[0]
            for q, (nx, ny) in zip(qs, shapes)]
    # FP32 on the component-wise scheme only: the reference's characteristic projection
    # (L R != I off rho = 1) amplifies FP32 rounding beyond the FP32 bound on these states
    for precision, tol in ((64, 1e-10), (32, 1e-5)) if cons else ((64, 1e-10),):
        b = wx.Batch(50000, 4, precision=precision, mode="fast", cons=cons, force_hlle=hlle, jp_cri=(0.05, 0.4),
                     cfl=0.45, tile_config=wx.Batch.STAGED)
        slots = [b.add(q, 1.0 / max(nx, ny), max_steps=6) for q, (nx, ny) in zip(qs, shapes)]
        b.run(7)
        for sl, ref in zip(slots, refs):
            assert b.info(sl)["steps"] == 6
            got = b.state(sl)
            for k in range(4):
                assert rel_l1(got[3:-3, 3:-3, k], ref[3:-3, 3:-3, k]) <= tol
        b.close()


def test_membership_changes(wx, orc):
    rng = np.random.default_rng(11)
    b = wx.Batch(100000, 4, precision=32, cons=True, force_hlle=False)
    qa = synced(orc, quadrant(rng, 30, 30))
    qb = synced(orc, quadrant(rng, 50, 20))
    a = b.add(qa, 1 / 30, max_steps=3)
    b.run(3)
    first = b.state(a)
    free0 = b.stats()["free_cells"]
    c = b.add(qb, 1 / 50, max_steps=6)
    assert b.stats()["free_cells"] < free0
    b.run(6)
    assert np.array_equal(b.state(a), first)  # finished solve untouched by the later run
    b.remove(a)
    d = b.add(qa, 1 / 30, max_steps=3)  # reuses the freed space
    b.run(3)
    assert np.array_equal(b.state(d), first)
    assert b.info(c)["steps"] == 6


def test_pool_full_and_slots(wx, orc):
    rng = np.random.default_rng(12)
    b = wx.Batch(3000, 2, precision=32)
    q = synced(orc, quadrant(rng, 40, 40))
    b.add(q, 1 / 40)
    with pytest.raises(ValueError):
        b.add(q, 1 / 40)  # pool of 3000 cells cannot hold two 1600-cell solves
    small = synced(orc, quadrant(rng, 10, 10))
    b.add(small, 0.1)
    with pytest.raises(ValueError):
        b.add(small, 0.1)  # both slots used


@pytest.mark.parametrize("precision", [32, 64])
def test_pool_cells_is_exact(wx, orc, precision):
    """Batch.pool_cells sizes a pool that holds exactly the given solves (rows padded
    to 16 bytes for the tile loads); one cell less does not."""
    rng = np.random.default_rng(13)
    shapes = [(37, 53), (64, 30), (19, 101)]  # row lengths not multiples of 16 bytes
    states = [synced(orc, quadrant(rng, nx, ny)) for nx, ny in shapes]
    cells = wx.Batch.pool_cells(shapes, precision)
    b = wx.Batch(cells, len(shapes), precision=precision, mode="fast")
    for (nx, ny), q in zip(shapes, states):
        b.add(q, 1.0 / max(nx, ny), max_steps=2)
    assert b.stats()["free_cells"] == 0
    b.run(2)
    for s in range(len(shapes)):
        assert b.info(s)["steps"] == 2 and b.info(s)["status"] == 0
    short = wx.Batch(cells - 16, len(shapes), precision=precision, mode="fast")
    with pytest.raises(ValueError):
        for (nx, ny), q in zip(shapes, states):
            short.add(q, 1.0 / max(nx, ny))


def test_staging_wait_runs_out(wx, orc):
    """A staging copy that never lands (the test hook does not issue it) makes its bounded
    wait give up: the CTA flags the solve of that tile and of every later tile it walks
    (WENO_ERR_CUDA, stopped), and the other solves' results are those of a clean run.
    Four solves on a fixed grid of 4 CTAs with 8 x 32 tiles: A (16 x 64) has tiles 0-3,
    B, C and D (8 x 32) one tile each (4, 5, 6); CTA 0 walks tiles 0 and 4."""
    rng = np.random.default_rng(41)
    shapes = [(16, 64), (8, 32), (8, 32), (8, 32)]
    qs = [synced(orc, quadrant(rng, nx, ny)) for nx, ny in shapes]
    kw = dict(precision=32, mode="fast", cons=True, force_hlle=True, cfl=0.45, tile_config=0)

    def batch():
        b = wx.Batch(20000, 4, **kw)
        return b, [b.add(q, 1.0 / max(nx, ny)) for q, (nx, ny) in zip(qs, shapes)]

    clean, cs = batch()
    clean.run(3)
    hooked, hs = batch()
    assert hooked.stats()["tiles"] == 7
    hooked.debug_skip_copy(0, wait_ns=2_000_000, grid=4)
    hooked.run(1)
    hooked.debug_skip_copy(-1)
    hooked.run(2)
    st = [hooked.info(s) for s in hs]
    assert [x["status"] for x in st] == [wx._lib.ERR_CUDA, wx._lib.ERR_CUDA, 0, 0]
    assert not st[0]["active"] and not st[1]["active"]
    assert st[0]["steps"] == 0 and st[1]["steps"] == 0
    for k in (2, 3):
        assert st[k]["steps"] == 3 and clean.info(cs[k])["status"] == 0
        assert np.array_equal(hooked.state(hs[k]), clean.state(cs[k]))
