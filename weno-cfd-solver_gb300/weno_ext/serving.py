"""Serving loop: continuous batching of solve requests on one GPU.

Requests arrive over time (a Poisson stream in the benchmark), each asking for
one problem (grid, initial data, end time) at FP32 or FP64.  The server keeps
one batched solver per precision, each with a fixed device pool carved from an
HBM budget.  A request is admitted as soon as its footprint (3 RK buffers x 4
conserved planes x its cells) fits in the free space of its pool and a slot is
free; until then it waits in arrival order.  Every loop iteration advances all
admitted solves of both pools by a few steps (the two pools run on their own
streams and overlap on the device), then retires the solves that reached their
end time, freeing their space for the next arrivals.  Time to solution is
measured from arrival to retirement.

Each solve's arithmetic depends only on its own state (tiles and the per-solve
dt reduction are independent of the other solves), so a result is bit-identical
alone and in the mix; tests/test_gpu_serving.py checks it.
"""

from __future__ import annotations

import dataclasses
import math
import time
from collections import deque

import numpy as np

from . import problems
from .batch import Batch


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the stream
    nx: int
    ny: int
    kind: str               # "quadrant" or "shock"
    precision: int          # 32 or 64
    t_end: float
    seed: int = 0
    mach: float = 10.0
    theta: float = math.pi / 3
    init: np.ndarray | None = None  # explicit (nx+6, ny+6, C) initial array (transmissive boundaries)
    # filled by the server
    admitted: float = float("nan")
    finished: float = float("nan")
    steps: int = 0
    t: float = 0.0
    status: int = 0
    slot: int = -1
    result: np.ndarray | None = None

    @property
    def cells(self):
        return self.nx * self.ny

    def build(self, device=True):
        """(q, dx, bc kwargs) of the request's initial data, generated on the GPU
        (device=True) or with the numpy generators."""
        if self.init is not None:
            return self.init, 1.0 / max(self.nx, self.ny), dict(bc="transmissive")
        if self.kind == "shock":
            lx, ly = self.nx / max(self.nx, self.ny), self.ny / max(self.nx, self.ny)
            gen = problems.oblique_shock_device if device else problems.oblique_shock
            q, bound, post = gen(self.nx, self.ny, lx, ly, self.mach, self.theta, x0=lx / 24)
            # the reference's oblique-shock driver steps at CFL 0.1 (double_mach_reflection.py:17)
            return q, lx / self.nx, dict(bc="dmr", bound=bound, post=post, cfl=0.1)
        gen = problems.quadrant_device if device else problems.quadrant
        return gen(self.nx, self.ny, seed=self.seed), 1.0 / max(self.nx, self.ny), dict(bc="transmissive")


CANCELLED = -1  # Request.status of a cancelled request (library status codes are >= 0)


def footprint_bytes(nx, ny, precision):
    es = 4 if precision == 32 else 8
    ld = -(-ny // (16 // es)) * (16 // es)  # rows padded to 16 bytes
    return 3 * 4 * (((nx * ld + 63) // 64) * 64) * es


def poisson_stream(n, rate, lo, hi, seed, fp64_fraction=0.25, t_end=(0.1, 0.3), shock_fraction=0.3):
    """Seeded requests: exponential inter-arrival times at `rate`/s, edges log-uniform
    in [lo, hi] (aspect <= 4), initial data quadrant or oblique shock, FP32 / FP64 tag."""
    rng = np.random.default_rng(seed)
    shapes = problems.batch_shapes(n, lo, hi, seed + 1)
    t = 0.0
    reqs = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        kind = "shock" if rng.random() < shock_fraction else "quadrant"
        reqs.append(Request(rid=k, arrival=t, nx=shapes[k][0], ny=shapes[k][1], kind=kind,
                            precision=64 if rng.random() < fp64_fraction else 32,
                            t_end=float(rng.uniform(*t_end)), seed=int(rng.integers(1 << 30)),
                            mach=float(rng.uniform(2.0, 10.0)), theta=math.radians(float(rng.uniform(30.0, 75.0)))))
    return reqs


class Server:
    def __init__(self, hbm_budget_bytes, *, fp64_share=0.5, max_solves=1024, steps_per_iter=8, cfl=0.5,
                 cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4), tile_config=(1, 1), keep_results=False):
        import torch
        self.torch = torch
        self.steps_per_iter = int(steps_per_iter)
        self.keep_results = keep_results
        b64 = int(hbm_budget_bytes * fp64_share)
        b32 = int(hbm_budget_bytes) - b64
        kw = dict(cons=cons, force_hlle=force_hlle, jp_cri=jp_cri, cfl=cfl)
        self.pools = {}
        self.budget = {32: b32, 64: b64}
        if b32 > 0:
            self.pools[32] = Batch(b32 // (3 * 4 * 4), max_solves, precision=32, mode="fast",
                                   tile_config=tile_config[0], **kw)
        if b64 > 0:
            self.pools[64] = Batch(b64 // (3 * 4 * 8), max_solves, precision=64, mode="fast",
                                   tile_config=tile_config[1], **kw)
        self.active = {p: {} for p in self.pools}  # slot -> request
        self.cancelled = set()  # request ids to drop (waiting) or stop (active)

    def cancel(self, rid):
        """Cancel request `rid`: dropped if it has not been admitted yet, otherwise
        stopped at the end of its pool's current chunk of steps (its slot and memory
        are freed then).  Its status becomes CANCELLED; the other requests are not
        affected.  May be called from the on_iteration callback."""
        self.cancelled.add(rid)

    def _admit(self, r, now):
        pool = self.pools.get(r.precision)
        if pool is None:
            raise ValueError(f"no pool for precision {r.precision}")
        q, dx, bc = r.build()
        try:
            r.slot = pool.add(q, dx, t_end=r.t_end, **bc)
        except ValueError:
            return False  # no space or no slot yet
        r.admitted = now
        self.active[r.precision][r.slot] = r
        return True

    def serve(self, requests, realtime=True, on_iteration=None, max_wall=None):
        """Run the stream to completion; returns the requests with timings filled in.

        Each pool is driven on its own: when its last chunk of steps has finished
        (a CUDA event on its stream), its finished solves are retired, waiting
        requests of its precision are admitted in arrival order, and the next chunk
        is enqueued.  realtime=False skips idle time to the next arrival."""
        torch = self.torch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting = {p: deque() for p in self.pools}
        for r in requests:
            if r.precision not in self.pools:
                raise ValueError(f"request {r.rid}: no pool for FP{r.precision}")
            if footprint_bytes(r.nx, r.ny, r.precision) > self.budget.get(r.precision, 0):
                raise ValueError(f"request {r.rid} ({r.nx}x{r.ny}, FP{r.precision}) exceeds its pool")
        inflight = {p: None for p in self.pools}
        t0 = time.perf_counter()
        iters = 0
        while pending or any(waiting[p] for p in self.pools) or any(self.active[p] for p in self.pools):
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                raise TimeoutError("serving loop exceeded max_wall")
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                waiting[r.precision].append(r)
            for p in self.pools:
                for r in [r for r in waiting[p] if r.rid in self.cancelled]:
                    waiting[p].remove(r)
                    r.finished, r.status = now, CANCELLED
            progressed = False
            for p, pool in self.pools.items():
                ev = inflight[p]
                if ev is not None and not ev.query():
                    continue
                if ev is not None or any(r.rid in self.cancelled for r in self.active[p].values()):
                    self._retire(p, time.perf_counter() - t0)
                    inflight[p] = None
                while waiting[p] and self._admit(waiting[p][0], time.perf_counter() - t0):
                    waiting[p].popleft()
                if self.active[p]:
                    pool.run(self.steps_per_iter)
                    ev = torch.cuda.Event()
                    ev.record(pool.stream)
                    inflight[p] = ev
                    progressed = True
                    iters += 1
            if on_iteration and progressed:
                on_iteration(iters, now)
            if not any(inflight.values()):
                if pending and not any(waiting[p] for p in self.pools):
                    wait = pending[0].arrival - (time.perf_counter() - t0)
                    if realtime:
                        time.sleep(max(0.0, min(wait, 0.01)))
                    else:
                        t0 -= max(0.0, wait)
            elif not progressed:
                time.sleep(0.0002)
        return requests

    def _retire(self, p, now):
        pool = self.pools[p]
        act, tt, nn = pool.poll()
        for slot, r in list(self.active[p].items()):
            if not act[slot] or r.rid in self.cancelled:
                inf = pool.info(slot)
                r.finished, r.steps, r.t = now, inf["steps"], inf["t"]
                r.status = CANCELLED if (act[slot] and r.rid in self.cancelled) else inf["status"]
                if self.keep_results:
                    r.result = pool.state(slot)
                pool.remove(slot)
                del self.active[p][slot]

    def close(self):
        for b in self.pools.values():
            b.close()


def summarize(requests, wall):
    tts = np.array([r.finished - r.arrival for r in requests if r.status == 0])
    cu = sum(r.cells * r.steps for r in requests)
    return {
        "requests": len(requests),
        "failed": sum(1 for r in requests if r.status not in (0, CANCELLED)),
        "cancelled": sum(1 for r in requests if r.status == CANCELLED),
        "p50_s": float(np.percentile(tts, 50)) if len(tts) else None,
        "p99_s": float(np.percentile(tts, 99)) if len(tts) else None,
        "mean_s": float(tts.mean()) if len(tts) else None,
        "cell_updates": int(cu),
        "wall_s": wall,
        "aggregate_cell_updates_per_s": cu / wall if wall > 0 else None,
        "fp64_requests": sum(1 for r in requests if r.precision == 64),
    }
