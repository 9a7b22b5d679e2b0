"""weno_l_local_noalloc: the residual with library-owned scratch, for callers that
cannot allocate device memory (a host that owns all device memory through its own
pool, a loop that must not pay cudaMalloc's device-wide synchronisation, code being
recorded into a CUDA graph).

The entry point is called through the C ABI and compared with weno_l_local (the
caller-workspace entry point) on the same inputs, in both arithmetic modes: the
two entry points run the same kernels, so the results must be bit-identical.  In
exact mode both are also compared with the oracle (the restated Rust core),
bit for bit -- the tolerance every exact-mode GPU test here uses.  Two calls in a
row check that the shared scratch array, which keeps the previous call's
contents, needs no clearing.  This file sorts last so that a run stopping at
the first failure has already run every other test; it also passes on its own in
a fresh process.
"""

import ctypes
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from states import quadrant  # noqa: E402

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20


def _load():
    from weno_ext import _lib
    return _lib, _lib.load()


def _call_both(L, _lib, torch, q, force_hlle, cons, jp=(0.05, 0.4), mode=None):
    mode = _lib.EXACT if mode is None else mode
    m, n, c = q.shape
    u = torch.from_numpy(q).cuda()
    s0, s1, s2 = u.stride()
    stream = torch.cuda.current_stream().cuda_stream
    dx = 1.0 / (m - 6)
    ref = torch.empty((m - 6, n - 6, 4), dtype=torch.float64, device="cuda")
    wsb = L.weno_l_local_workspace(m, n, force_hlle)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(L.weno_l_local(u.data_ptr(), m, n, c, s0, s1, s2, dx, 1.4, force_hlle, jp[0], jp[1], cons,
                              mode, ref.data_ptr(), ws.data_ptr(), wsb, stream), "weno_l_local")
    outs = []
    for _ in range(2):
        out = torch.full((m - 6, n - 6, 4), float("nan"), dtype=torch.float64, device="cuda")
        rc = L.weno_l_local_noalloc(u.data_ptr(), m, n, c, s0, s1, s2, dx, 1.4, force_hlle, jp[0], jp[1], cons,
                                    mode, out.data_ptr(), stream)
        _lib.check(rc, "weno_l_local_noalloc")
        outs.append(out.cpu().numpy())
    return ref.cpu().numpy(), outs


@pytest.mark.parametrize("force_hlle,cons,nx,ny", [(1, 0, 200, 150), (0, 1, 96, 130), (0, 0, 500, 520),
                                                   (1, 1, 700, 700)])
def test_noalloc_matches_caller_workspace(force_hlle, cons, nx, ny):
    import torch
    _lib, L = _load()
    m, n = nx + 6, ny + 6
    assert L.weno_l_local_workspace(m, n, force_hlle) <= SCRATCH_BYTES
    q = quadrant(np.random.default_rng(nx + ny), nx, ny)
    ref, outs = _call_both(L, _lib, torch, q, force_hlle, cons)
    for got in outs:
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("force_hlle,cons", [(1, 0), (0, 0), (0, 1), (1, 1)])
def test_noalloc_matches_oracle(force_hlle, cons):
    """Exact mode against the oracle, bit for bit, on a non-square four-quadrant state."""
    import torch
    from oracle import oracle
    _lib, L = _load()
    nx, ny = 72, 57
    q = quadrant(np.random.default_rng(5 + force_hlle + 2 * cons), nx, ny)
    ref = oracle.l_local_py(q, 1.0 / nx, 1.4, bool(force_hlle), (0.05, 0.4), bool(cons))
    dev_ref, outs = _call_both(L, _lib, torch, q, force_hlle, cons)
    assert np.array_equal(dev_ref, ref)
    for got in outs:
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("force_hlle,cons", [(1, 0), (0, 0), (1, 1)])
def test_noalloc_fast_mode(force_hlle, cons):
    """FAST mode through the same entry point: bit-identical to weno_l_local in FAST mode
    (the same kernels) and within 1e-11 of the largest magnitude of the oracle's result."""
    import torch
    from oracle import oracle
    _lib, L = _load()
    nx, ny = 150, 96
    q = quadrant(np.random.default_rng(17 + force_hlle + 2 * cons), nx, ny)
    ref, outs = _call_both(L, _lib, torch, q, force_hlle, cons, mode=_lib.FAST)
    exact = oracle.l_local_py(q, 1.0 / nx, 1.4, bool(force_hlle), (0.05, 0.4), bool(cons))
    assert np.abs(ref - exact).max() <= 1e-11 * np.abs(exact).max()
    for got in outs:
        assert np.array_equal(got, ref)


def test_noalloc_calls_of_different_sizes_in_a_row():
    """A large call leaves its data in the shared scratch; a smaller one after it
    must not read any of it."""
    import torch
    _lib, L = _load()
    big = quadrant(np.random.default_rng(1), 520, 500)
    small = quadrant(np.random.default_rng(2), 40, 33)
    for q, hlle in ((big, 0), (small, 0), (small, 1), (big, 1)):
        ref, outs = _call_both(L, _lib, torch, q, hlle, 0)
        for got in outs:
            assert np.array_equal(got, ref)


def test_noalloc_rejects_sizes_beyond_the_scratch():
    import torch
    _lib, L = _load()
    m = n = 1030
    assert L.weno_l_local_workspace(m, n, 1) > SCRATCH_BYTES
    u = torch.ones((m, n, 4), dtype=torch.float64, device="cuda")
    out = torch.zeros((m - 6, n - 6, 4), dtype=torch.float64, device="cuda")
    rc = L.weno_l_local_noalloc(u.data_ptr(), m, n, 4, n * 4, 4, 1, 0.01, 1.4, 1, 0.2, 1.0, 0, _lib.EXACT,
                                out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.ERR_WORKSPACE
    assert b"scratch" in L.weno_last_error()
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0  # nothing was launched
