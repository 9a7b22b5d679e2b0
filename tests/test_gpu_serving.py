"""Serving loop: continuous batching with HBM-footprint admission.  Each result must
be bit-identical alone and in the mix; FP64 results (exact slabs) equal the oracle bit
for bit and FP32 ones agree within 1e-5 relative L1; admission never exceeds the
budget, does not block small requests behind a large one, holds them back once the
large one has waited past the age bound, and hands emptied slabs to the precision
with a backlog; a request with non-finite initial data finishes with a numeric
status without disturbing the others; a request larger than a slab is refused up
front."""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(wx, r):
    from weno_ext import serving
    solo = serving.Request(**{k: getattr(r, k) for k in ("rid", "arrival", "nx", "ny", "kind", "precision", "t_end",
                                                         "seed", "mach", "theta", "init")})
    solo.arrival = 0.0
    srv = serving.Server(64 << 20, max_solves=4, steps_per_iter=3, keep_results=True)
    srv.serve([solo], realtime=False, max_wall=120)
    srv.close()
    return solo


def test_stream_results_equal_alone(wx):
    from weno_ext import serving
    reqs = serving.poisson_stream(14, rate=400.0, lo=24, hi=72, seed=5, fp64_fraction=0.3, t_end=(0.01, 0.03),
                                  shock_fraction=0.3)
    budget = 3 << 20  # small: forces requests to wait for space
    srv = serving.Server(budget, slabs=2, max_solves=16, steps_per_iter=4, keep_results=True)
    peak = [0]

    def watch(it, now):
        peak[0] = max(peak[0], sum(sl.used for sl in srv.slabs))
        for sl in srv.slabs:
            if sl.batch is not None:
                es = 4 if sl.precision == 32 else 8
                cap = sl.nbytes // (3 * 4 * es)
                assert 3 * 4 * es * (cap - sl.batch.stats()["free_cells"]) <= sl.nbytes + 3 * 4 * es * 16

    srv.serve(reqs, realtime=False, on_iteration=watch, max_wall=300)
    srv.close()
    assert all(r.status == 0 and r.finished >= r.arrival for r in reqs)
    assert all(abs(r.t - r.t_end) < 1e-9 for r in reqs)
    assert any(r.admitted > r.arrival for r in reqs)  # some had to wait
    assert 0 < peak[0] <= budget
    summary = serving.summarize(reqs, max(r.finished for r in reqs))
    assert summary["failed"] == 0 and summary["p99_s"] >= summary["p50_s"]
    for r in (reqs[0], reqs[5], reqs[-1]):
        solo = _alone(wx, r)
        assert solo.steps == r.steps and solo.t == r.t
        assert np.array_equal(solo.result, r.result)


def test_nan_request_fails_alone(wx):
    from weno_ext import problems, serving
    good = serving.Request(rid=0, arrival=0.0, nx=40, ny=40, kind="quadrant", precision=32, t_end=0.02, seed=1)
    q = problems.quadrant(40, 40, seed=2)
    q[20, 20, 0] = float("nan")
    bad = serving.Request(rid=1, arrival=0.0, nx=40, ny=40, kind="quadrant", precision=32, t_end=0.02, init=q)
    srv = serving.Server(16 << 20, max_solves=4, steps_per_iter=4, keep_results=True)
    srv.serve([good, bad], realtime=False, max_wall=120)
    srv.close()
    assert good.status == 0 and bad.status != 0
    solo = _alone(wx, good)
    assert np.array_equal(solo.result, good.result)


def test_oversized_request_is_refused(wx):
    from weno_ext import serving
    r = serving.Request(rid=0, arrival=0.0, nx=512, ny=512, kind="quadrant", precision=64, t_end=0.01)
    srv = serving.Server(8 << 20, max_solves=2)
    with pytest.raises(ValueError):
        srv.serve([r], realtime=False)
    srv.close()


def test_cancel_active_and_waiting_requests(wx):
    """A request cancelled while on the GPU is stopped at the end of its pool's chunk
    and one cancelled while waiting is never admitted; both end CANCELLED, and the
    others finish with results equal to their runs alone."""
    from weno_ext import serving
    reqs = [serving.Request(rid=k, arrival=0.0, nx=48, ny=40, kind="quadrant", precision=32, t_end=0.03, seed=k)
            for k in range(5)]
    budget = serving.footprint_bytes(48, 40, 32) * 2 + 4096  # two at a time: the rest wait
    srv = serving.Server(budget, slabs=1, max_solves=4, steps_per_iter=2, keep_results=True)
    seen = {}

    def on_iteration(it, now):
        if it == 1:
            active = [r.rid for r in srv.active[32].values()]
            seen["active"] = active[0]
            srv.cancel(active[0])
            srv.cancel(4)  # still waiting: the pool holds two solves

    srv.serve(reqs, realtime=False, on_iteration=on_iteration, max_wall=120)
    srv.close()
    stopped = reqs[seen["active"]]
    assert stopped.status == serving.CANCELLED and 0 < stopped.steps and stopped.t < stopped.t_end
    assert reqs[4].status == serving.CANCELLED and reqs[4].steps == 0 and math.isnan(reqs[4].admitted)
    done = [r for r in reqs if r.rid not in (seen["active"], 4)]
    assert all(r.status == 0 and abs(r.t - r.t_end) < 1e-9 for r in done)
    summary = serving.summarize(reqs, 1.0)
    assert summary["cancelled"] == 2 and summary["failed"] == 0
    solo = _alone(wx, done[0])
    assert np.array_equal(solo.result, done[0].result)


def _oracle_solve(orc, r):
    """The oracle's driver loop for a quadrant request, from the state the batched solver
    starts from (boundary fill, primitive sync), to the request's t_end."""
    from test_gpu_batch import synced
    from test_gpu_solver import oracle_run
    from weno_ext import problems
    q = synced(orc, problems.quadrant(r.nx, r.ny, seed=r.seed))
    ref, T, steps = oracle_run(orc, q, r.nx, r.ny, 1.0 / max(r.nx, r.ny), 0.5, 10 ** 6, t_final=r.t_end,
                               jp=(1e4, 1.1e4), cons=True, hlle=False)
    return ref, T, steps


def test_served_results_match_oracle(wx, orc):
    """FP64 requests on exact slabs equal the oracle's driver loop bit for bit; FP32
    requests agree with it within 1e-5 relative L1 in every conserved variable."""
    from states import rel_l1
    from weno_ext import serving
    reqs = [serving.Request(rid=0, arrival=0.0, nx=40, ny=56, kind="quadrant", precision=64, t_end=0.03, seed=3),
            serving.Request(rid=1, arrival=0.0, nx=64, ny=33, kind="quadrant", precision=32, t_end=0.03, seed=4),
            serving.Request(rid=2, arrival=0.001, nx=50, ny=50, kind="quadrant", precision=64, t_end=0.02, seed=5),
            serving.Request(rid=3, arrival=0.002, nx=37, ny=70, kind="quadrant", precision=32, t_end=0.02, seed=6)]
    srv = serving.Server(64 << 20, slabs=4, max_solves=8, steps_per_iter=3, keep_results=True, fp64_mode="exact")
    srv.serve(reqs, realtime=False, max_wall=120)
    srv.close()
    for r in reqs:
        ref, T, steps = _oracle_solve(orc, r)
        assert r.status == 0 and r.steps == steps
        if r.precision == 64:
            assert r.t == T
            assert np.array_equal(r.result, ref)
        else:
            assert abs(r.t - T) <= 1e-6 * T
            for k in range(4):
                assert rel_l1(r.result[3:-3, 3:-3, k], ref[3:-3, 3:-3, k]) <= 1e-5


def test_small_request_passes_a_waiting_large_one(wx):
    """One slab that holds the first request and a small one, but not the large one:
    the small request behind the large one is admitted while the large one waits."""
    from weno_ext import serving
    fp = serving.footprint_bytes
    small = dict(nx=40, ny=40, kind="quadrant", precision=32, t_end=0.05)
    a = serving.Request(rid=0, arrival=0.0, seed=1, **small)
    big = serving.Request(rid=1, arrival=0.0005, nx=96, ny=96, kind="quadrant", precision=32, t_end=0.01, seed=2)
    c = serving.Request(rid=2, arrival=0.001, seed=3, **small)
    budget = fp(96, 96, 32) + fp(40, 40, 32) // 2  # a + c fit; a + big do not
    srv = serving.Server(budget, slabs=1, max_solves=4, steps_per_iter=2)
    srv.serve([a, big, c], realtime=True, max_wall=120)
    srv.close()
    assert all(r.status == 0 for r in (a, big, c))
    assert c.admitted < big.admitted


def test_age_bound_holds_back_younger_requests(wx):
    """With an age bound of zero the large request at the head is starving at once:
    the small request behind it is not admitted before it."""
    from weno_ext import serving
    fp = serving.footprint_bytes
    small = dict(nx=40, ny=40, kind="quadrant", precision=32, t_end=0.05)
    a = serving.Request(rid=0, arrival=0.0, seed=1, **small)
    big = serving.Request(rid=1, arrival=0.0005, nx=96, ny=96, kind="quadrant", precision=32, t_end=0.01, seed=2)
    c = serving.Request(rid=2, arrival=0.001, seed=3, **small)
    budget = fp(96, 96, 32) + fp(40, 40, 32) // 2
    srv = serving.Server(budget, slabs=1, max_solves=4, steps_per_iter=2, max_wait_s=0.0)
    srv.serve([a, big, c], realtime=True, max_wall=120)
    srv.close()
    assert all(r.status == 0 for r in (a, big, c))
    assert c.admitted >= big.admitted


def test_slabs_follow_the_backlog(wx):
    """Two slabs, both taken by FP32 requests; FP64 requests that arrive later get a slab
    once one has emptied (handed over to FP64), and every request finishes."""
    from weno_ext import serving
    reqs = [serving.Request(rid=k, arrival=0.0, nx=40, ny=40, kind="quadrant", precision=32,
                            t_end=0.01 * (1 + k), seed=k) for k in range(4)]
    reqs += [serving.Request(rid=4 + k, arrival=0.0, nx=40, ny=40, kind="quadrant", precision=64, t_end=0.01,
                             seed=10 + k) for k in range(2)]
    slab = serving.footprint_bytes(40, 40, 64) + 1024  # one FP64 or two FP32 requests per slab
    # fused batches for both precisions, so that a request's slab bytes are its state pools
    srv = serving.Server(2 * slab, slabs=2, max_solves=4, steps_per_iter=2, max_wait_s=0.0, tile_config=(1, 1))
    srv.serve(reqs, realtime=False, max_wall=120)
    srv.close()
    assert all(r.status == 0 and abs(r.t - r.t_end) < 1e-9 for r in reqs)
    assert srv.conversions >= 1
    assert min(r.admitted for r in reqs[4:]) >= min(r.finished for r in reqs[:4])


def test_adaptive_chunks_keep_results(wx):
    """Chunks sized by measured GPU time (chunk_ms) change only when requests are
    serviced: every request still reaches its t_end with the result it has alone."""
    from weno_ext import serving
    reqs = serving.poisson_stream(10, rate=300.0, lo=24, hi=80, seed=9, fp64_fraction=0.3, t_end=(0.01, 0.03),
                                  shock_fraction=0.3)
    srv = serving.Server(8 << 20, slabs=2, max_solves=16, steps_per_iter=2, keep_results=True, chunk_ms=2.0)
    srv.serve(reqs, realtime=False, max_wall=300)
    chunks = [sl.chunk for sl in srv.slabs]
    srv.close()
    assert all(r.status == 0 and abs(r.t - r.t_end) < 1e-9 for r in reqs)
    assert any(c > 0 for c in chunks)
    for r in (reqs[1], reqs[-2]):
        solo = _alone(wx, r)
        assert solo.steps == r.steps and np.array_equal(solo.result, r.result)
