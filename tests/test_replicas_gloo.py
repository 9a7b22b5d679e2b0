"""The N>1 bench path (independent replicas): barrier, max-over-ranks timing and
the whole-job rate, on two gloo ranks on CPU."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from weno_ext import replicas
    replicas.init("gloo")
    w, r, lr = replicas.world()
    replicas.barrier()
    ms = replicas.max_over_ranks(100.0 + 50.0 * r)  # rank 1 is the slow one
    out[r] = (w, ms, replicas.job_rate(1000, ms, w))
    replicas.finish()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    w, ms, rate = res[0]
    assert w == 2 and ms == 150.0
    assert rate == pytest.approx(2 * 1000 / 0.150)


def test_single_process_defaults(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from weno_ext import replicas
    assert replicas.world() == (1, 0, 0)
    assert replicas.max_over_ranks(3.5) == 3.5
