"""The serving loop's admission policy on the CPU, with a stand-in batch: no head-of-line
blocking, the age bound, slabs changing precision with the backlog, slab accounting
within the budget, and cancellation.  (The GPU tests run the same policy on real
batches: tests/test_gpu_serving.py.)"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "weno-cfd-solver_gb300"))

from weno_ext import serving  # noqa: E402


class _Event:
    def record(self, stream):
        pass

    def query(self):
        return True

    def elapsed_time(self, other):
        return 1.0


class _Cuda:
    Event = staticmethod(lambda enable_timing=False: _Event())
    Stream = staticmethod(lambda priority=0: None)


class _Torch:
    cuda = _Cuda()


class FakeBatch:
    """Pool of `pool_cells` cells; a solve needs cells = footprint / (12 es) and
    finishes after round(t_end * 1000) steps."""

    opened = []

    def __init__(self, pool_cells, max_solves, *, precision, mode, tile_config, **kw):
        self.capacity, self.max_solves, self.precision = int(pool_cells), int(max_solves), precision
        self.solves = {}
        self.stream = None
        FakeBatch.opened.append(self)

    def add(self, q, dx, *, t_end=None, **bc):
        nx, ny = q.shape[0] - 6, q.shape[1] - 6
        need = serving.footprint_bytes(nx, ny, self.precision) // (12 * (4 if self.precision == 32 else 8))
        used = sum(s["cells"] for s in self.solves.values())
        if used + need > self.capacity or len(self.solves) >= self.max_solves:
            raise ValueError("full")
        slot = min(set(range(self.max_solves)) - set(self.solves))
        self.solves[slot] = {"cells": need, "steps": 0, "goal": max(1, round(t_end * 1000)), "t_end": t_end}
        return slot

    def run(self, n):
        for s in self.solves.values():
            s["steps"] = min(s["goal"], s["steps"] + n)

    def poll(self):
        act = np.zeros(self.max_solves, dtype=bool)
        for k, s in self.solves.items():
            act[k] = s["steps"] < s["goal"]
        return act, None, None

    def info(self, slot):
        s = self.solves[slot]
        done = s["steps"] >= s["goal"]
        return {"t": s["t_end"] if done else 0.0, "steps": s["steps"], "active": not done, "status": 0}

    def state(self, slot):
        return np.zeros(1)

    def remove(self, slot):
        del self.solves[slot]

    def close(self):
        pass

    @staticmethod
    def bytes_per_cell(precision, force_hlle=False, tile_config=1):
        return 12.0 * (4 if precision == 32 else 8)


@pytest.fixture
def fake(monkeypatch):
    """Server factory whose slabs hold FakeBatch pools and whose chunks complete at once."""
    monkeypatch.setattr(serving, "Batch", FakeBatch)
    FakeBatch.opened = []

    def make(budget, **kw):
        srv = serving.Server(budget, **kw)
        srv.torch = _Torch()
        return srv
    return make


def _req(rid, arrival, n, precision, t_end):
    q = np.zeros((n + 6, n + 6, 8))
    return serving.Request(rid=rid, arrival=arrival, nx=n, ny=n, kind="quadrant", precision=precision,
                           t_end=t_end, init=q)


def test_no_head_of_line_blocking(fake):
    fp = serving.footprint_bytes
    a, big, c = _req(0, 0.0, 40, 32, 0.05), _req(1, 0.0, 96, 32, 0.01), _req(2, 0.0, 40, 32, 0.05)
    srv = fake(fp(96, 96, 32) + fp(40, 40, 32) // 2, slabs=1, max_solves=4, steps_per_iter=2)
    srv.serve([a, big, c], realtime=False)
    assert all(r.status == 0 and r.t == r.t_end for r in (a, big, c))
    assert c.admitted <= big.admitted and a.admitted <= big.admitted
    assert big.admitted >= max(a.finished, c.finished) - 1e-9


def test_age_bound_holds_younger_requests(fake):
    fp = serving.footprint_bytes
    a, big, c = _req(0, 0.0, 40, 32, 0.05), _req(1, 0.0, 96, 32, 0.01), _req(2, 0.0, 40, 32, 0.05)
    srv = fake(fp(96, 96, 32) + fp(40, 40, 32) // 2, slabs=1, max_solves=4, steps_per_iter=2, max_wait_s=0.0)
    srv.serve([a, big, c], realtime=False)
    assert all(r.status == 0 for r in (a, big, c))
    assert c.admitted >= big.admitted


def test_slab_changes_precision_with_the_backlog(fake):
    fp = serving.footprint_bytes
    reqs = [_req(k, 0.0, 40, 32, 0.01 * (1 + k)) for k in range(4)] + [_req(4 + k, 0.0, 40, 64, 0.01)
                                                                       for k in range(2)]
    slab = fp(40, 40, 64) + 1024  # one FP64 or two FP32 requests per slab
    srv = fake(2 * slab, slabs=2, max_solves=4, steps_per_iter=2, max_wait_s=0.0)
    srv.serve(reqs, realtime=False)
    assert all(r.status == 0 and r.t == r.t_end for r in reqs)
    assert srv.conversions >= 1
    assert min(r.admitted for r in reqs[4:]) >= min(r.finished for r in reqs[:4])
    assert sum(1 for b in FakeBatch.opened if b.precision == 64) >= 1


def test_slab_accounting_stays_within_the_budget(fake):
    rng = np.random.default_rng(3)
    reqs = [_req(k, float(rng.uniform(0, 0.01)), int(rng.integers(8, 48)), int(rng.choice([32, 64])),
                 float(rng.uniform(0.005, 0.03))) for k in range(40)]
    budget = 900_000  # three slabs, each above the largest FP64 request (48 x 48: 221 KB)
    srv = fake(budget, slabs=3, max_solves=8, steps_per_iter=3)
    peak = [0]

    def watch(it, now):
        peak[0] = max(peak[0], sum(sl.used for sl in srv.slabs))
        for sl in srv.slabs:
            assert 0 <= sl.used <= sl.nbytes

    srv.serve(reqs, realtime=False, on_iteration=watch)
    assert all(r.status == 0 and r.t == r.t_end for r in reqs)
    assert 0 < peak[0] <= budget
    assert all(sl.used == 0 for sl in srv.slabs)


def test_cancel_waiting_request(fake):
    fp = serving.footprint_bytes
    reqs = [_req(k, 0.0, 40, 32, 0.02) for k in range(3)]
    srv = fake(fp(40, 40, 32) + 1024, slabs=1, max_solves=4, steps_per_iter=2)

    def on_iteration(it, now):
        if it == 1:
            srv.cancel(2)

    srv.serve(reqs, realtime=False, on_iteration=on_iteration)
    assert reqs[2].status == serving.CANCELLED and reqs[2].steps == 0
    assert reqs[0].status == 0 and reqs[1].status == 0
