"""Tile-shape autotuner of the batched solver.

The batched solver has five compiled tile configurations: four shapes of the
fused stage kernel (TX x TY interior cells per CTA, with a 3-cell halo -- 4
with the sensor blend -- staged in shared memory) and the staged kernels
(three launches per stage, the faces in a device workspace, no halo
recompute).  Which one is fastest depends on the precision (shared memory per
CTA and hence residency; in FP64 the staged kernels win, the halo recompute
costing more than the traffic it saves), the scheme (register pressure of the
characteristic projection, the blend's extra halo) and the mix of grid sizes
(partial tiles at the edges of small grids).  `best_tile_config` times every
configuration on the caller's batch for a few graph-replayed steps and caches
the winner per (GPU, precision, arithmetic, scheme, size class).
"""

from __future__ import annotations

import json
import math
import os

from . import _lib

_DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_build",
                              "autotune.json")


def cache_path():
    return os.environ.get("WENO_AUTOTUNE_CACHE", _DEFAULT_CACHE)


def size_class(shapes):
    """Geometric-mean edge rounded to a power of two (64, 128, ..., 4096)."""
    g = math.exp(sum(math.log(max(1, nx * ny)) for nx, ny in shapes) / (2 * len(shapes)))
    return int(2 ** round(math.log2(max(g, 1.0))))


def _key(precision, mode, cons, force_hlle, shapes):
    import torch
    name = torch.cuda.get_device_name().replace(" ", "_")
    return f"{name}|p{precision}|{mode}|{'cons' if cons else 'char'}|{'hlle' if force_hlle else 'blend'}|" \
           f"e{size_class(shapes)}"


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def measure(states, *, precision, mode, cons, force_hlle, jp_cri, cfl, gamma=1.4, steps=3, warmup=1):
    """Milliseconds per step of every tile configuration on a batch of `states`
    [(q, dx), ...]; configurations that do not fit are reported as None."""
    import torch
    from .batch import Batch
    cells = Batch.pool_cells([(q.shape[0] - 6, q.shape[1] - 6) for q, _ in states], precision)
    times = {}
    for cfg in range(_lib.load().weno_batch_tile_config_count()):
        try:
            b = Batch(cells, len(states), precision=precision, mode=mode, cons=cons,
                      force_hlle=force_hlle, jp_cri=jp_cri, gamma=gamma, cfl=cfl, tile_config=cfg)
        except ValueError:
            times[cfg] = None
            continue
        for q, dx in states:
            b.add(q, dx)
        b.run(warmup)
        b.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(b.stream)
        b.run(steps)
        e1.record(b.stream)
        e1.synchronize()
        times[cfg] = e0.elapsed_time(e1) / steps
        b.close()
    return times


def best_tile_config(states, *, precision, mode="fast", cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4), cfl=0.5,
                     gamma=1.4, refresh=False):
    """The fastest tile configuration for this kind of batch (cached)."""
    shapes = [(q.shape[0] - 6, q.shape[1] - 6) for q, _ in states]
    key = _key(precision, mode, cons, force_hlle, shapes)
    cache = _load()
    if not refresh and key in cache:
        return int(cache[key]["config"]), cache[key]
    times = measure(states, precision=precision, mode=mode, cons=cons, force_hlle=force_hlle, jp_cri=jp_cri,
                    cfl=cfl, gamma=gamma)
    valid = {k: v for k, v in times.items() if v is not None}
    best = min(valid, key=valid.get)
    entry = {"config": best, "ms_per_step": {str(k): v for k, v in times.items()}}
    cache[key] = entry
    _store(cache)
    return best, entry
