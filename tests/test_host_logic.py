"""Host-side logic that needs no GPU: request streams, pool sizing, admission
footprints, the serving summary, problem generators and the autotuner's cache."""

import json
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "weno-cfd-solver_gb300"))

from weno_ext import autotune, problems, serving  # noqa: E402
from weno_ext.batch import Batch  # noqa: E402


def test_poisson_stream_is_seeded_and_ordered():
    a = serving.poisson_stream(50, rate=20.0, lo=128, hi=2048, seed=7)
    b = serving.poisson_stream(50, rate=20.0, lo=128, hi=2048, seed=7)
    c = serving.poisson_stream(50, rate=20.0, lo=128, hi=2048, seed=8)
    key = lambda rs: [(r.arrival, r.nx, r.ny, r.kind, r.precision, r.t_end, r.seed) for r in rs]  # noqa: E731
    assert key(a) == key(b) and key(a) != key(c)
    arr = [r.arrival for r in a]
    assert arr == sorted(arr) and arr[0] > 0
    assert all(128 <= min(r.nx, r.ny) and max(r.nx, r.ny) <= 2048 for r in a)
    assert all(max(r.nx, r.ny) / min(r.nx, r.ny) <= 4.0 for r in a)
    assert {r.precision for r in a} <= {32, 64} and {r.kind for r in a} <= {"quadrant", "shock"}
    assert all(2.0 <= r.mach <= 10.0 and math.radians(30) <= r.theta <= math.radians(75) for r in a)


@pytest.mark.parametrize("precision,q", [(32, 4), (64, 2)])
def test_pool_cells_and_footprint_agree(precision, q):
    shapes = [(37, 53), (64, 30), (19, 101), (128, 128)]
    es = 4 if precision == 32 else 8
    cells = Batch.pool_cells(shapes, precision)
    expect = 0
    for nx, ny in shapes:
        ld = -(-ny // q) * q
        assert ld % q == 0 and ld >= ny and (ld * es) % 16 == 0
        plane = ((nx * ld + 63) // 64) * 64
        expect += plane
        assert serving.footprint_bytes(nx, ny, precision) == 3 * 4 * plane * es
    assert cells == expect


def test_summarize_counts_failures_and_cancellations():
    R = serving.Request
    reqs = [R(rid=k, arrival=0.0, nx=10, ny=10, kind="quadrant", precision=32, t_end=0.1) for k in range(5)]
    for k, r in enumerate(reqs):
        r.finished, r.steps = 1.0 + k, 10
    reqs[3].status = 5                   # numeric failure
    reqs[4].status = serving.CANCELLED
    s = serving.summarize(reqs, wall=2.0)
    assert s["requests"] == 5 and s["failed"] == 1 and s["cancelled"] == 1
    assert s["p50_s"] == pytest.approx(2.0) and s["p99_s"] <= 3.0
    assert s["cell_updates"] == 5 * 100 * 10 and s["aggregate_cell_updates_per_s"] == pytest.approx(2500.0)


def test_rankine_hugoniot_and_oblique_shock_generator():
    rho, u, v, p = problems.rankine_hugoniot(10.0, math.pi / 3)
    assert rho == pytest.approx(8.0, abs=1e-12) and p == pytest.approx(116.5, abs=1e-12)
    assert math.hypot(u, v) == pytest.approx(8.25, rel=1e-12)
    q, bound, post = problems.oblique_shock(40, 10, 4.0, 1.0, 10.0, math.pi / 3)
    assert q.shape == (46, 16, 8) and post.shape == (8,)
    # conserved channels consistent with the primitive ones everywhere
    r, uu, vv, pp = q[..., 4], q[..., 5], q[..., 6], q[..., 7]
    assert np.allclose(q[..., 1], r * uu) and np.allclose(q[..., 2], r * vv)
    assert np.allclose(q[..., 3], pp / 0.4 + 0.5 * r * (uu * uu + vv * vv))
    assert 3 <= bound < 46


def test_quadrant_generator_states():
    st = problems.quadrant_states(11)
    q = problems.quadrant(30, 20, seed=11)
    assert len(st) == 4
    for rho, u, v, p in st:
        assert 0.1 <= rho <= 2.0 and 0.1 <= p <= 2.0 and -1 <= u <= 1 and -1 <= v <= 1
    rho0, u0, v0, p0 = st[0]
    assert q[3, 3, 4] == rho0 and q[3, 3, 7] == p0 and q[3, 3, 1] == rho0 * u0


def test_batch_shapes_respect_range_and_aspect():
    shapes = problems.batch_shapes(200, 64, 1024, 5)
    assert len(shapes) == 200
    assert all(64 <= min(s) and max(s) <= 1024 and max(s) / min(s) <= 4.0 for s in shapes)


def test_autotune_size_class_and_cache(tmp_path, monkeypatch):
    assert autotune.size_class([(64, 64)]) == 64
    assert autotune.size_class([(1024, 1024), (1024, 1024)]) == 1024
    assert autotune.size_class([(100, 400)]) == 256  # geometric-mean edge 200 -> 256
    monkeypatch.setenv("WENO_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    autotune._store({"k": {"config": 2}})
    assert json.loads((tmp_path / "tune.json").read_text()) == {"k": {"config": 2}}
    assert autotune._load() == {"k": {"config": 2}}
    (tmp_path / "tune.json").write_text("not json")
    assert autotune._load() == {}


def test_batch_bytes_per_cell():
    """Memory a pool cell costs: the three RK pools of four planes, plus the staged
    configuration's workspace share (1.25 x (16 + 2 NF) values, NF = 4 HLLE / 9 blend)."""
    assert Batch.bytes_per_cell(32, False, 1) == 12 * 4
    assert Batch.bytes_per_cell(64, True, 0) == 12 * 8
    assert Batch.bytes_per_cell(64, True, Batch.STAGED) == (12 + 1.25 * 24) * 8
    assert Batch.bytes_per_cell(64, False, Batch.STAGED) == (12 + 1.25 * 34) * 8
