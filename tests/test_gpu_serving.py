"""Serving loop: continuous batching with HBM-footprint admission.  Each result must
be bit-identical alone and in the mix; admission never exceeds the budget; a request
with non-finite initial data finishes with a numeric status without disturbing the
others; a request larger than its pool is refused up front."""

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
    srv = serving.Server(budget, max_solves=16, steps_per_iter=4, keep_results=True)
    peak = {32: 0, 64: 0}

    cells = {p: srv.budget[p] // (3 * 4 * (4 if p == 32 else 8)) for p in srv.pools}

    def watch(it, now):
        for p, b in srv.pools.items():
            peak[p] = max(peak[p], cells[p] - b.stats()["free_cells"])

    srv.serve(reqs, realtime=False, on_iteration=watch, max_wall=300)
    srv.close()
    assert all(r.status == 0 and r.finished >= r.arrival for r in reqs)
    assert all(abs(r.t - r.t_end) < 1e-9 for r in reqs)
    assert any(r.admitted > r.arrival for r in reqs)  # some had to wait
    for p in peak:
        assert 0 < peak[p] <= cells[p] + 16  # the pool is the budget (capacity rounded up to 64 elements)
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
    srv = serving.Server(2 * budget, fp64_share=0.5, max_solves=4, steps_per_iter=2, keep_results=True)
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
