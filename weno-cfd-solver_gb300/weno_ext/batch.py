"""Batched solver: many independent problems of uneven size stepped together.

Each solve runs the reference drivers' loop (Rie_prob_2d_rs.py:169-207,
311-365 with transmissive boundaries, or double_mach_reflection.py:97-134 with
the oblique-shock boundary of unitest.py:207-227) with its own dt and end time.
All active solves advance together: one step is five kernel launches whatever
the number of solves (per-solve dt, three fused stage kernels walking a packed
tile list, clock update), replayed from a captured CUDA graph.  Solves join and
leave between runs, which is what the serving loop builds on.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .solver import DMR_POST


class Batch:
    def __init__(self, pool_cells, max_solves, *, precision=32, mode="fast", cons=True, force_hlle=False,
                 jp_cri=(1e4, 1.1e4), gamma=1.4, cfl=0.5, tile_config=1, stream=None, weno_eps=1e-12):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("Batch needs a CUDA GPU; there is no CPU fallback")
        self._torch = torch
        self.L = _lib.load()
        self.max_solves = int(max_solves)
        self.precision = int(precision)
        self.gamma = float(gamma)
        self.stream = stream if stream is not None else torch.cuda.Stream()
        h = ctypes.c_void_p()
        _lib.check(self.L.weno_batch_create(
            ctypes.byref(h), int(pool_cells), self.max_solves, self.precision,
            _lib.FAST if mode == "fast" else _lib.EXACT, int(bool(cons)), int(bool(force_hlle)), self.gamma,
            float(jp_cri[0]), float(jp_cri[1]), float(cfl), float(weno_eps), int(tile_config), self.stream.cuda_stream),
            "Batch")
        self._h = h
        self.shapes = {}

    @staticmethod
    def pool_cells(shapes, precision=32):
        """Pool size (cells) that holds solves of the given (nx, ny) shapes at once:
        rows padded to 16 bytes, each plane rounded up to 64 elements."""
        q = 16 // (4 if int(precision) == 32 else 8)
        return sum(((nx * (-(-ny // q) * q) + 63) // 64) * 64 for nx, ny in shapes)

    @staticmethod
    def tile_configs():
        return _lib.load().weno_batch_tile_config_count()

    # tile configuration of the staged kernels (three launches per stage, faces in a workspace)
    STAGED = 4

    @staticmethod
    def bytes_per_cell(precision=32, force_hlle=False, tile_config=1):
        """Device bytes one pool cell costs (the three RK pools, plus the staged
        configuration's share of the face workspace)."""
        return _lib.load().weno_batch_bytes_per_cell(int(precision), int(bool(force_hlle)), int(tile_config))

    def add(self, q, dx, *, t_end=None, max_steps=None, bc="transmissive", bound=0, post=None, cfl=None):
        """Add a solve from its (nx+6, ny+6, C>=4) array (numpy or torch CUDA); returns its slot."""
        torch = self._torch
        if not isinstance(q, torch.Tensor):
            q = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float64)).to(self.stream.device if hasattr(
                self.stream, "device") else "cuda")
        if q.dtype != torch.float64 or q.dim() != 3:
            raise TypeError("state must be a 3-D float64 array")
        self.stream.wait_stream(torch.cuda.current_stream())
        M, N, C = q.shape
        post8 = np.ascontiguousarray(DMR_POST if post is None else post, dtype=np.float64)
        slot = ctypes.c_int()
        s = q.stride()
        _lib.check(self.L.weno_batch_add(
            self._h, M - 6, N - 6, float(dx), {"transmissive": _lib.BC_TRANSMISSIVE, "dmr": _lib.BC_DMR}[bc],
            int(bound), post8.ctypes.data, -1.0 if t_end is None else float(t_end),
            0 if max_steps is None else int(max_steps), -1.0 if cfl is None else float(cfl), q.data_ptr(), C, s[0],
            s[1], s[2], ctypes.byref(slot)),
            "batch add")
        self.shapes[slot.value] = (M - 6, N - 6)
        return slot.value

    def remove(self, slot):
        _lib.check(self.L.weno_batch_remove(self._h, int(slot)), "batch remove")
        self.shapes.pop(slot, None)

    def run(self, nsteps, graph=True):
        _lib.check(self.L.weno_batch_run(self._h, int(nsteps), int(bool(graph))), "batch run")

    def state(self, slot, device=False):
        torch = self._torch
        nx, ny = self.shapes[slot]
        out = torch.empty((nx + 6, ny + 6, 8), dtype=torch.float64, device="cuda")
        _lib.check(self.L.weno_batch_get_state(self._h, int(slot), out.data_ptr()), "batch state")
        return out if device else out.cpu().numpy()

    def info(self, slot):
        t = ctypes.c_double()
        n = ctypes.c_int64()
        a = ctypes.c_int()
        st = ctypes.c_int()
        _lib.check(self.L.weno_batch_info(self._h, int(slot), ctypes.byref(t), ctypes.byref(n), ctypes.byref(a),
                                          ctypes.byref(st)), "batch info")
        return {"t": t.value, "steps": n.value, "active": bool(a.value), "status": st.value}

    def poll(self):
        """(active, t, steps) arrays over all slots, after synchronising."""
        a = np.zeros(self.max_solves, dtype=np.int32)
        t = np.zeros(self.max_solves)
        n = np.zeros(self.max_solves, dtype=np.int64)
        _lib.check(self.L.weno_batch_poll(self._h, a.ctypes.data, t.ctypes.data, n.ctypes.data), "batch poll")
        return a.astype(bool), t, n

    def stats(self):
        nt = ctypes.c_int64()
        fc = ctypes.c_int64()
        lp = ctypes.c_int()
        _lib.check(self.L.weno_batch_stats(self._h, ctypes.byref(nt), ctypes.byref(fc), ctypes.byref(lp)), "stats")
        return {"tiles": nt.value, "free_cells": fc.value, "launches_per_step": lp.value}

    def debug_skip_copy(self, tile, wait_ns=2_000_000, grid=0):
        """Test hook of the bounded TMA waits: later runs do not issue the staging copy of
        packed tile `tile` (its wait gives up after `wait_ns`); `grid` > 0 fixes the stage
        kernels' persistent grid.  tile < 0 restores normal operation."""
        _lib.check(self.L.weno_batch_debug_skip_copy(self._h, int(tile), int(wait_ns), int(grid)), "debug_skip_copy")

    def synchronize(self):
        self.stream.synchronize()

    def close(self):
        if getattr(self, "_h", None):
            self.L.weno_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
