"""Serving loop: continuous batching of solve requests on one GPU.

Requests arrive over time (a Poisson stream in the benchmark), each asking for
one problem (grid, initial data, end time) at FP32 or FP64.  The HBM budget is
divided into slabs; a slab holds one batched solver (weno_ext.Batch) of one
precision, created when the slab is first needed.  A request is admitted as
soon as its footprint (3 RK buffers x 4 conserved planes x its cells) fits in a
slab of its precision, or in a free slab, which then takes that precision.
Slabs follow the backlog: a slab whose solves have all retired is handed to
the other precision when requests of that precision are waiting and fit
nowhere, so the FP32/FP64 split is not fixed.

Admission scans the waiting requests in arrival order and admits every one
that fits (a large request at the head does not block smaller ones behind
it).  An age bound keeps large requests from starving: once the oldest waiting
request of a precision has waited longer than ``max_wait_s``, younger requests
of that precision are held back until it is admitted.

Each slab is driven on its own stream: when its last chunk of steps has
finished (a CUDA event), its finished solves are retired, admission runs, and
the next chunk is enqueued, so the slabs' work overlaps on the device.  Time to
solution is measured from arrival to retirement.

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


class _Slab:
    __slots__ = ("index", "nbytes", "precision", "batch", "active", "inflight", "used", "draining", "chunk",
                 "t_start", "steps")

    def __init__(self, index, nbytes):
        self.index = index
        self.nbytes = nbytes
        self.precision = None  # 32 or 64 once a batch lives here
        self.batch = None
        self.active = {}  # slot -> request
        self.inflight = None  # CUDA event of the last enqueued chunk
        self.used = 0  # footprint bytes of the admitted requests
        self.draining = False  # takes no new requests: it is being emptied for the other precision
        self.chunk = 0  # steps of the next chunk (0: the server's initial chunk)
        self.t_start = None  # CUDA event at the start of the chunk in flight
        self.steps = 0  # steps of the chunk in flight

    def fits(self, r, need):
        return self.nbytes - self.used >= need


class Server:
    """Continuous-batching server over an HBM budget of `hbm_budget_bytes` split into
    `slabs` slabs.  `steps_per_iter`: steps of a slab's first chunk (and of every chunk
    when `chunk_ms` is None); `tile_config`: the batch configuration of (FP32, FP64)
    slabs; `keep_results`: True keeps every finished request's array in
    `Request.result`, a set of request ids keeps those only; `max_wait_s`: the age bound
    of admission; `fp64_mode`: "fast" or "exact" arithmetic of the FP64 slabs.  The
    scheme arguments (`cfl`, `cons`, `force_hlle`, `jp_cri`) apply to every request."""

    def __init__(self, hbm_budget_bytes, *, slabs=4, max_solves=1024, steps_per_iter=8, cfl=0.5, cons=True,
                 force_hlle=False, jp_cri=(1e4, 1.1e4), tile_config=(1, Batch.STAGED), keep_results=False,
                 max_wait_s=None, fp64_mode="fast", chunk_ms=None):
        import torch
        self.torch = torch
        self.steps_per_iter = int(steps_per_iter)
        # chunk_ms: size each slab's chunk of steps to about this much GPU time (measured
        # on its last chunk), so newly arrived requests wait about that long for a slab
        # whatever its load; None keeps steps_per_iter steps per chunk.
        self.chunk_ms = chunk_ms
        self.keep_results = keep_results
        self.max_wait_s = max_wait_s
        self.max_solves = int(max_solves)
        self.fp64_mode = fp64_mode
        # tile configuration per precision: the fused tile kernel for FP32, the staged
        # kernels for FP64 (bound by the FP64 pipe, where recomputing halo faces
        # costs more than moving the faces through HBM)
        self.tile_config = {32: tile_config[0], 64: tile_config[1]}
        # device bytes per pool cell of each precision's batches, against the 3 x 4
        # state values per cell that footprint_bytes counts
        self.scale = {p: Batch.bytes_per_cell(p, force_hlle, self.tile_config[p]) / (12 * (4 if p == 32 else 8))
                      for p in (32, 64)}
        self.kw = dict(cons=cons, force_hlle=force_hlle, jp_cri=jp_cri, cfl=cfl)
        n = max(1, int(slabs))
        self.slab_bytes = int(hbm_budget_bytes) // n
        self.slabs = [_Slab(k, self.slab_bytes) for k in range(n)]
        self.cancelled = set()  # request ids to drop (waiting) or stop (active)
        self.conversions = 0  # slabs handed from one precision to the other

    # -- views by precision ---------------------------------------------------
    @property
    def active(self):
        """{precision: {(slab, slot): request}} of the admitted requests."""
        out = {32: {}, 64: {}}
        for sl in self.slabs:
            if sl.precision:
                for slot, r in sl.active.items():
                    out[sl.precision][(sl.index, slot)] = r
        return out

    @property
    def pools(self):
        """{precision: [Batch, ...]} of the slabs that hold a batch."""
        out = {}
        for sl in self.slabs:
            if sl.batch is not None:
                out.setdefault(sl.precision, []).append(sl.batch)
        return out

    def cancel(self, rid):
        """Cancel request `rid`: dropped if it has not been admitted yet, otherwise
        stopped at the end of its slab's current chunk of steps (its slot and memory
        are freed then).  Its status becomes CANCELLED; the other requests are not
        affected.  May be called from the on_iteration callback."""
        self.cancelled.add(rid)

    # -- slabs ----------------------------------------------------------------
    def need(self, r):
        """Bytes request `r` takes in a slab: its state pools and, for a staged
        batch, its face workspace."""
        return int(math.ceil(footprint_bytes(r.nx, r.ny, r.precision) * self.scale[r.precision]))

    def _open(self, sl, precision):
        mode = "fast" if precision == 32 else self.fp64_mode
        cfg = self.tile_config[precision]
        bpc = Batch.bytes_per_cell(precision, self.kw["force_hlle"], cfg)
        # FP32 slabs on a high-priority stream: their requests need about 30x less
        # time per cell than FP64 ones, and the block scheduler then places their
        # CTAs ahead of the FP64 slab's queued ones
        stream = self.torch.cuda.Stream(priority=-1) if precision == 32 else None
        sl.batch = Batch(int(sl.nbytes // bpc), self.max_solves, precision=precision, mode=mode, tile_config=cfg,
                         stream=stream, **self.kw)
        sl.precision = precision

    def _release(self, sl):
        sl.batch.close()
        sl.batch = None
        sl.precision = None
        sl.active = {}
        sl.inflight = None
        sl.used = 0
        sl.draining = False
        sl.chunk = 0

    def _try_add(self, sl, r, now):
        q, dx, bc = r.build()
        try:
            r.slot = sl.batch.add(q, dx, t_end=r.t_end, **bc)
        except ValueError:
            return False  # no space (first-fit fragmentation) or no slot in this slab
        r.admitted = now
        sl.active[r.slot] = r
        sl.used += self.need(r)
        return True

    def _place(self, r, now):
        """Admit `r`: into an idle slab of its precision with room; if every slab of its
        precision with room is busy, it waits for them (no new slab is opened); else into
        a free slab, or into an idle, empty slab of the other precision, which changes
        precision.  Returns "admitted", "busy" or "full"."""
        need = self.need(r)
        mine = [sl for sl in self.slabs if sl.precision == r.precision and not sl.draining and sl.fits(r, need)]
        for sl in mine:
            if sl.inflight is None and self._try_add(sl, r, now):
                return "admitted"
        if any(sl.inflight is not None for sl in mine):
            return "busy"
        for sl in self.slabs:
            if sl.precision is None:
                self._open(sl, r.precision)
                return "admitted" if self._try_add(sl, r, now) else "full"
        for sl in self.slabs:
            if sl.precision not in (None, r.precision) and not sl.active and sl.inflight is None:
                self._release(sl)
                self.conversions += 1
                self._open(sl, r.precision)
                return "admitted" if self._try_add(sl, r, now) else "full"
        return "full"

    def _admit_waiting(self, waiting, now):
        held = set()  # precisions whose oldest request has waited past the age bound
        for r in list(waiting):
            if r.precision in held:
                continue
            res = self._place(r, now)
            if res == "admitted":
                waiting.remove(r)
                continue
            if self.max_wait_s is not None and now - r.arrival > self.max_wait_s:
                held.add(r.precision)
                if res == "full" and not any(sl.draining for sl in self.slabs):
                    # no slab of its precision can take it: empty the other precision's
                    # least-loaded slab so it can change hands
                    other = [sl for sl in self.slabs if sl.precision not in (None, r.precision)]
                    if other:
                        min(other, key=lambda sl: sl.used).draining = True

    def serve(self, requests, realtime=True, on_iteration=None, max_wall=None):
        """Run the stream to completion; returns the requests with timings filled in.

        A slab is serviced when its last chunk of steps has finished: its finished
        solves are retired, waiting requests are admitted (every one that fits, in
        arrival order, subject to the age bound), and its next chunk is enqueued.
        realtime=False skips idle time to the next arrival."""
        torch = self.torch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting = []
        for r in requests:
            if r.precision not in (32, 64):
                raise ValueError(f"request {r.rid}: precision must be 32 or 64")
            if self.need(r) > self.slab_bytes:
                raise ValueError(f"request {r.rid} ({r.nx}x{r.ny}, FP{r.precision}) exceeds a slab of "
                                 f"{self.slab_bytes} bytes")
        t0 = time.perf_counter()
        iters = 0
        while pending or waiting or any(sl.active for sl in self.slabs):
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                raise TimeoutError("serving loop exceeded max_wall")
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            for r in [r for r in waiting if r.rid in self.cancelled]:
                waiting.remove(r)
                r.finished, r.status = now, CANCELLED
            # retire on every slab whose chunk is done
            for sl in self.slabs:
                if sl.inflight is not None and sl.inflight.query():
                    if self.chunk_ms is not None:
                        per_step = sl.t_start.elapsed_time(sl.inflight) / max(sl.steps, 1)
                        sl.chunk = int(min(64, max(1, round(self.chunk_ms / max(per_step, 1e-3)))))
                    sl.inflight = None
                    self._retire(sl, time.perf_counter() - t0)
                elif sl.inflight is None and any(r.rid in self.cancelled for r in sl.active.values()):
                    self._retire(sl, time.perf_counter() - t0)
            if waiting:
                self._admit_waiting(waiting, time.perf_counter() - t0)
            progressed = False
            for sl in self.slabs:
                if sl.inflight is None and sl.active:
                    timing = self.chunk_ms is not None
                    sl.steps = sl.chunk or self.steps_per_iter
                    if timing:
                        sl.t_start = torch.cuda.Event(enable_timing=True)
                        sl.t_start.record(sl.batch.stream)
                    sl.batch.run(sl.steps)
                    ev = torch.cuda.Event(enable_timing=timing)
                    ev.record(sl.batch.stream)
                    sl.inflight = ev
                    progressed = True
                    iters += 1
            if on_iteration and progressed:
                on_iteration(iters, now)
            if not any(sl.inflight is not None for sl in self.slabs):
                if pending and not waiting:
                    wait = pending[0].arrival - (time.perf_counter() - t0)
                    if realtime:
                        time.sleep(max(0.0, min(wait, 0.01)))
                    else:
                        t0 -= max(0.0, wait)
            elif not progressed:
                time.sleep(0.0002)
        return requests

    def _retire(self, sl, now):
        pool = sl.batch
        act, tt, nn = pool.poll()
        for slot, r in list(sl.active.items()):
            if not act[slot] or r.rid in self.cancelled:
                inf = pool.info(slot)
                r.finished, r.steps, r.t = now, inf["steps"], inf["t"]
                r.status = CANCELLED if (act[slot] and r.rid in self.cancelled) else inf["status"]
                keep = self.keep_results
                if keep is True or (isinstance(keep, (set, frozenset)) and r.rid in keep):
                    r.result = pool.state(slot)
                pool.remove(slot)
                del sl.active[slot]
                sl.used -= self.need(r)

    def close(self):
        for sl in self.slabs:
            if sl.batch is not None:
                self._release(sl)


def summarize(requests, wall):
    tts = np.array([r.finished - r.arrival for r in requests if r.status == 0])
    cu = sum(r.cells * r.steps for r in requests)
    per = {}
    for p in (32, 64):
        t = np.array([r.finished - r.arrival for r in requests if r.status == 0 and r.precision == p])
        w = np.array([r.admitted - r.arrival for r in requests if r.status == 0 and r.precision == p])
        if len(t):
            per[f"fp{p}"] = {"requests": int(len(t)), "p50_s": float(np.percentile(t, 50)),
                             "p99_s": float(np.percentile(t, 99)), "p50_queue_s": float(np.percentile(w, 50)),
                             "p99_queue_s": float(np.percentile(w, 99)),
                             "cell_updates": int(sum(r.cells * r.steps for r in requests if r.precision == p))}
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
        "by_precision": per,
    }
