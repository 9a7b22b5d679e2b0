#!/usr/bin/env python3
"""Benchmark of the GB300 2D Euler step: cell-updates/s of SSP-RK3 steps.

Workload (default): the 4096 x 4096 four-quadrant Riemann problem (seeded
rho, p ~ U[0.1, 2], u, v ~ U[-1, 1] per quadrant, gamma = 1.4, 3 ghost cells,
transmissive boundaries), characteristic WENO5 + 2-point Gauss-quadrature faces
+ HLLE, CFL 0.45, FP64.  One step = one full SSP-RK3 step (three residual
evaluations, stage combinations, boundary fills and the CFL reduction) over
all nx*ny cells; one cell-update = one cell advanced one step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

gb300 arm: the device-resident solver (weno_ext.Solver, C ABI of
libweno_gb300.so) with the state resident in HBM; `value` is whole-job
cell-updates/s over the K timed steps (CUDA events on the solver's stream,
barrier + synchronize on both sides, max over ranks).  `e2e` is the same metric
through the public API with host buffers: every step copies the (nx+6, ny+6, 8)
state in from pinned host memory and the result back.  Under torchrun each rank
runs an independent replica (the path does not shard here).

reference arm: the reference's CPU implementation of the path -- the oracle's
C++ restatement of the Rust core and driver step (the Rust crate cannot be
built without a Rust toolchain) -- on all host cores, on a bounded strip of
the same workload per step.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "weno-cfd-solver_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

GAMMA = 1.4
SEED = 20261203
METRIC = "cell-updates/s (4096^2 four-quadrant Riemann, char-WENO5+GQ+HLLE, SSP-RK3, FP64)"
UNIT = "cell-updates/s"
# Kernel classes reported by weno_solver_timing_report.
CLASSES = ["cfl+dt", "bc", "pass1_x", "pass2_x", "blend", "pass1_y", "pass2_y", "residual+rk"]


def quadrant_state(nx, ny, seed=SEED):
    from weno_ext import problems
    return problems.quadrant(nx, ny, seed=seed)


def load_json(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, watts, reasons = [], [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            try:
                watts.append(float(parts[3]))
            except ValueError:
                pass
            for nm, val in zip(names[1:], parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w": statistics.median(watts) if watts else None}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(nx, strip_ny, threads, seconds_hint=10.0):
    """The oracle (C++ restatement of the Rust core and driver step) timed on host
    cores over a strip of the workload: nx x strip_ny interior cells."""
    from oracle import oracle
    used = oracle.set_threads(threads)
    q = quadrant_state(nx, strip_ny, seed=SEED + 1)
    oracle.bc_transmissive(q)
    dx = 1.0 / nx
    dt = 0.45 * dx / oracle.cfl_cmax(q, nx, strip_ny, GAMMA)
    t0 = time.perf_counter()
    steps = 0
    while True:
        oracle.rk3_step(q, nx, strip_ny, dx, dt, GAMMA, True, (0.2, 1.0), False)
        steps += 1
        if time.perf_counter() - t0 >= seconds_hint or steps >= 400:
            break
    el = time.perf_counter() - t0
    line = {"value": nx * strip_ny * steps / el, "unit": UNIT, "cores": used, "kind": "port",
            "sample": f"{steps} SSP-RK3 step(s) of a {nx} x {strip_ny} strip of the same workload "
                      f"(oracle C++ restatement, OpenMP, {used} threads), {el:.1f} s"}
    # The reference's Rust core is single-threaded: the same restatement on one core.
    oracle.set_threads(1)
    q1 = quadrant_state(nx, 4, seed=SEED + 1)
    oracle.bc_transmissive(q1)
    dt1 = 0.45 * dx / oracle.cfl_cmax(q1, nx, 4, GAMMA)
    t0 = time.perf_counter()
    steps1 = 0
    while True:
        oracle.rk3_step(q1, nx, 4, dx, dt1, GAMMA, True, (0.2, 1.0), False)
        steps1 += 1
        if time.perf_counter() - t0 >= seconds_hint / 2 or steps1 >= 400:
            break
    el1 = time.perf_counter() - t0
    oracle.set_threads(used)
    line["single_core"] = {"value": nx * 4 * steps1 / el1, "unit": UNIT, "cores": 1,
                           "sample": f"{steps1} step(s) of a {nx} x 4 strip, one thread (the reference's Rust "
                                     f"core is single-threaded), {el1:.1f} s"}
    return line


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    nx = args.nx
    # Bounded sample: a strip of the workload sized for a few seconds per step.
    strip = int(os.environ.get("WENO_REF_STRIP", "48"))
    from oracle import oracle
    used = oracle.set_threads(nthreads)
    q = quadrant_state(nx, strip, seed=SEED + 1)
    oracle.bc_transmissive(q)
    dx = 1.0 / nx
    for _ in range(args.warmup):
        dt = 0.45 * dx / oracle.cfl_cmax(q, nx, strip, GAMMA)
        oracle.rk3_step(q, nx, strip, dx, dt, GAMMA, True, (0.2, 1.0), False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt = 0.45 * dx / oracle.cfl_cmax(q, nx, strip, GAMMA)
        oracle.rk3_step(q, nx, strip, dx, dt, GAMMA, True, (0.2, 1.0), False)
    el = time.perf_counter() - t0
    value = nx * strip * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"four-quadrant Riemann {nx}x{args.ny} (timed on a {nx}x{strip} strip per step), "
                               "char-WENO5+GQ+HLLE, SSP-RK3, CFL 0.45", "nx": nx, "ny": args.ny,
                   "sample_ny": strip},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": used, "kind": "port",
                         "sample": f"{args.steps} step(s) of a {nx} x {strip} strip, oracle C++ restatement of "
                                   f"the Rust core (Rust toolchain absent), OpenMP {used} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _l1_linf(a, b):
    out = {}
    for k, nm in enumerate(("rho", "rho_u", "rho_v", "E")):
        x, y = a[3:-3, 3:-3, k], b[3:-3, 3:-3, k]
        den = np.abs(y).sum()
        out[nm] = {"rel_l1": float(np.abs(x - y).sum() / den) if den else None,
                   "linf": float(np.abs(x - y).max()),
                   "rel_linf": float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))}
    return out


def _lockstep(nx, ny, dx, q0, kw, runs, checkpoints):
    """Run the solvers of `runs` [(name, precision, mode)] side by side from q0, timing
    each on its own stream; returns per-run timings and, at every checkpoint, the
    L1/Linf of each run against the first one."""
    import torch
    import weno_ext
    sol = {}
    for name, prec, mode in runs:
        s = weno_ext.Solver(nx, ny, dx, GAMMA, precision=prec, mode=mode, **kw)
        s.set_state(q0)
        sol[name] = s
    ms = {name: 0.0 for name in sol}
    tot0 = {name: s.totals() for name, s in sol.items()}
    errs, done = [], 0
    ref = runs[0][0]
    for c in checkpoints:
        for name, s in sol.items():
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s.stream)
            s.run(c - done)
            e1.record(s.stream)
            e1.synchronize()
            ms[name] += e0.elapsed_time(e1)
        done = c
        st = {name: s.state() for name, s in sol.items()}
        errs.append({"step": c, **{name: _l1_linf(st[name], st[ref]) for name in st if name != ref}})
    res = {}
    for name, s in sol.items():
        t, k, status = s.info()
        res[name] = {"steps": k, "t": t, "status": status, "ms_per_step": ms[name] / max(done, 1),
                     "cell_updates_per_s": nx * ny * k / (ms[name] / 1e3) if ms[name] else None,
                     "totals_start": tot0[name], "totals_end": s.totals()}
        s.close()
    return res, errs


def _first_nonfinite(nx, ny, dx, q0, kw, nsteps, mode):
    """First step after which the state holds a non-finite value (None if none within nsteps)."""
    import weno_ext
    s = weno_ext.Solver(nx, ny, dx, GAMMA, precision=64, mode=mode, **kw)
    s.set_state(q0)
    blow = None
    for k in range(1, nsteps + 1):
        s.run(1)
        if not all(math.isfinite(x) for x in s.totals()):
            blow = k
            break
    s.close()
    return blow


def run_accuracy(args):
    """Accuracy of FP32 and FP64-fast against exact FP64 (bit-identical to the reference's
    arithmetic) per configuration, in both reconstructions:

    c1: 2048^2 four-quadrant (seeded rho, p ~ U[0.1,2], u, v ~ U[-1,1]), WENO5 + GQ + HLLE,
        CFL 0.45; c2: oblique shock 4096x1024 on [0,4]x[0,1], seeded Mach ~ U[2,10] and
        angle ~ U[30,75] deg, WENO5 + GQ + HLLC (blend 1e4/1.1e4), CFL 0.1, with the
        oblique-shock inflow / outflow / reflecting-wall boundary.

    The configurations name the characteristic reconstruction.  With the reference's
    eigenvector matrices (its left eigenvectors carry 0.5/(rho c), so L R != I off
    rho = 1) that scheme turns non-finite on both problems in exact FP64, i.e. in the
    reference's own arithmetic; it is run up to the last finite step, and the
    component-wise reconstruction for the configured step count (500 / 1000)."""
    import torch
    torch.cuda.set_device(0)
    from weno_ext import problems
    if args.config == "c1":
        nx, ny, nsteps = 2048, 2048, int(os.environ.get("WENO_C1_STEPS", "500"))
        q0 = problems.quadrant(nx, ny, seed=SEED + 1)
        kw = dict(force_hlle=True, jp_cri=(0.2, 1.0), cfl=0.45)
        dx, extra = 1.0 / 2048, {}
        desc = f"four-quadrant Riemann {nx}x{ny}, WENO5+GQ+HLLE, CFL 0.45"
    else:
        nx, ny, nsteps = 4096, 1024, int(os.environ.get("WENO_C2_STEPS", "1000"))
        rng = np.random.default_rng(SEED + 2)
        mach, theta = float(rng.uniform(2, 10)), math.radians(float(rng.uniform(30, 75)))
        q0, bound, post = problems.oblique_shock(nx, ny, 4.0, 1.0, mach, theta)
        kw = dict(force_hlle=False, jp_cri=(1e4, 1.1e4), cfl=0.1, bc="dmr", bound=bound, post=post)
        dx, extra = 1.0 / 1024, {"mach": mach, "theta_deg": math.degrees(theta), "bound": bound}
        desc = (f"oblique shock {nx}x{ny} on [0,4]x[0,1], M={mach:.3f}, angle={math.degrees(theta):.2f} deg, "
                "WENO5+GQ+HLLC(blend 1e4/1.1e4), CFL 0.1")
    runs = (("fp64_exact", 64, "exact"), ("fp64_fast", 64, "fast"), ("fp32", 32, "fast"))
    out = {}
    blow = _first_nonfinite(nx, ny, dx, q0, dict(kw, cons=False), nsteps, "exact")
    char_steps = nsteps if blow is None else blow - 1
    marks = sorted({max(1, char_steps * f // 4) for f in (1, 2, 3, 4)})
    res, errs = _lockstep(nx, ny, dx, q0, dict(kw, cons=False), runs, marks)
    out["characteristic"] = {"steps": char_steps, "first_nonfinite_step_fp64_exact": blow, "runs": res,
                             "errors_vs_fp64_exact": errs}
    res, errs = _lockstep(nx, ny, dx, q0, dict(kw, cons=True), runs,
                          sorted({nsteps * f // 4 for f in (1, 2, 3, 4)}))
    out["component_wise"] = {"steps": nsteps, "runs": res, "errors_vs_fp64_exact": errs}
    line = {"metric": "accuracy and cell-updates/s", "config_name": args.config, "unit": UNIT, "n_gpus": 1,
            "data": "synthetic", "config": dict({"workload": desc}, **extra), **out}
    print(json.dumps(line))
    return 0


def batched_accuracy(nsolves, every=16):
    """FP32 batched solves against FP64 (fast arithmetic, within 1e-10 of the reference's)
    runs of the same solves: every `every`-th solve of the batched workload, to t_end."""
    import weno_ext
    from weno_ext import problems
    rng = np.random.default_rng(SEED + 3)
    shapes = problems.batch_shapes(nsolves, 64, 1024, SEED + 3)
    t_ends = rng.uniform(0.1, 0.3, len(shapes))
    pick = list(range(0, len(shapes), every))
    states = {k: (problems.quadrant(*shapes[k], seed=SEED + k), 1.0 / max(shapes[k])) for k in pick}
    kw = dict(mode="fast", cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4), cfl=0.5)
    results = {}
    for prec in (32, 64):
        b = weno_ext.Batch(weno_ext.Batch.pool_cells([shapes[k] for k in pick], prec), len(pick), precision=prec,
                           **kw)
        slots = {k: b.add(states[k][0], states[k][1], t_end=float(t_ends[k])) for k in pick}
        while b.poll()[0].any():
            b.run(50)
        results[prec] = {k: (b.info(sl), b.state(sl)) for k, sl in slots.items()}
        b.close()
    per, l1, linf = [], [], []
    for k in pick:
        i32, s32 = results[32][k]
        i64, s64 = results[64][k]
        if i32["status"] or i64["status"]:
            per.append({"solve": k, "shape": shapes[k], "status": [i32["status"], i64["status"]]})
            continue
        e = _l1_linf(s32, s64)
        l1.append(e["rho"]["rel_l1"])
        linf.append(e["rho"]["rel_linf"])
        per.append({"solve": k, "shape": shapes[k], "steps": [i32["steps"], i64["steps"]],
                    "rho_rel_l1": e["rho"]["rel_l1"], "rho_rel_linf": e["rho"]["rel_linf"]})
    return {"solves_compared": len(l1), "rho_rel_l1_max": max(l1) if l1 else None,
            "rho_rel_l1_median": float(np.median(l1)) if l1 else None,
            "rho_rel_linf_max": max(linf) if linf else None, "per_solve": per,
            "reference": "FP64 batch, fast arithmetic (within 1e-10 relative L1 of exact FP64)"}


def batched_leg(nsolves, tune=True, tile_config=None, precision=32, max_steps=None):
    """Batched: independent four-quadrant solves of uneven size (edges log-uniform in
    [64, 1024], aspect <= 4), each with its own dt and t_end ~ U[0.1, 0.3], component
    WENO5 + HLLC (blend thresholds 1e4 / 1.1e4), FP32, CFL 0.5, all advanced together by
    graph-replayed steps of the persistent tile kernels; the tile shape is autotuned.
    Solves that reach t_end leave the batch between chunks of steps, so the tile list
    holds only active solves.  Returns the result as a dict."""
    import torch
    torch.cuda.set_device(0)
    import weno_ext
    from weno_ext import autotune, problems
    rng = np.random.default_rng(SEED + 3)
    shapes = problems.batch_shapes(nsolves, 64, 1024, SEED + 3)
    states = [(problems.quadrant(nx, ny, seed=SEED + k), 1.0 / max(nx, ny)) for k, (nx, ny) in enumerate(shapes)]
    t_ends = rng.uniform(0.1, 0.3, len(shapes))
    kw = dict(precision=precision, mode="fast", cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4), cfl=0.5)
    sample = states[:: max(1, len(states) // 64)]
    if tile_config is not None:
        cfg, tuning = int(tile_config), None
    elif tune:
        cfg, tuning = autotune.best_tile_config(sample, **kw)
    else:
        cfg, tuning = 1, None
    cells = sum(nx * ny for nx, ny in shapes)
    b = weno_ext.Batch(weno_ext.Batch.pool_cells(shapes, precision), len(shapes), tile_config=cfg, **kw)
    slots = [b.add(q, dx, t_end=float(te), max_steps=max_steps) for (q, dx), te in zip(states, t_ends)]
    ntiles0 = b.stats()["tiles"]
    b.run(1)
    b.synchronize()
    done_before = b.poll()[2].copy()
    chunk = 20 if max_steps is None else max(1, min(20, max_steps - 1))
    final = {}
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # steady state: every solve active (no solve finishes within the first chunk)
    es0 = torch.cuda.Event(enable_timing=True)
    es1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(b.stream)
    es0.record(b.stream)
    b.run(chunk)
    es1.record(b.stream)
    graph_steps = chunk
    while True:
        act, tt, nn = b.poll()
        for k, sl in enumerate(slots):
            if k not in final and not act[sl]:
                final[k] = (b.info(sl), int(nn[sl]))
                b.remove(sl)
        if len(final) == len(slots):
            break
        b.run(chunk)
        graph_steps += chunk
    e1.record(b.stream)
    e1.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    steady_ms = es0.elapsed_time(es1)
    steps = np.array([final[k][1] for k in range(len(slots))])
    cu = int(sum(nx * ny * (int(n) - int(done_before[sl])) for (nx, ny), n, sl in zip(shapes, steps, slots)))
    st = b.stats()
    # Solves the reference scheme itself drives non-finite (component-wise WENO5 has no
    # positivity limiter) stop with a numeric status; the others must reach t_end.
    failed = [k for k in range(len(slots)) if final[k][0]["status"] != 0]
    ok = [k for k in range(len(slots)) if k not in set(failed)]
    tt = np.array([final[k][0]["t"] for k in range(len(slots))])
    b.close()
    pname = "FP32" if precision == 32 else "FP64 (fast arithmetic)"
    return {
        "metric": f"aggregate cell-updates/s, batched uneven four-quadrant solves ({pname})",
        "value": cu / (ms / 1e3), "unit": UNIT, "dtype": "f32" if precision == 32 else "f64",
        "config": {"workload": f"{len(shapes)} four-quadrant solves, edges log-uniform [64,1024], aspect<=4, "
                               f"cons-WENO5+GQ+HLLC, {pname}, CFL 0.5, t_end~U[0.1,0.3], per-solve dt"
                               + (f", at most {max_steps} steps per solve" if max_steps else ""),
                   "cells": cells, "tiles": ntiles0, "tile_config": cfg, "autotune": tuning},
        "steady_state": {"ms_per_step": steady_ms / chunk, "cell_updates_per_s": cells * chunk / (steady_ms / 1e3),
                         "note": f"the first {chunk} graph-replayed steps, every solve active"},
        "steps_replayed": graph_steps, "cell_updates": cu, "gpu_ms": ms, "wall_s": wall,
        "launches_per_step": st["launches_per_step"],
        "max_steps_of_a_solve": int(steps.max()), "min_steps_of_a_solve": int(steps.min()),
        "solves_nonfinite": len(failed),
        "t_end_reached_by_the_others": bool(np.all(np.abs(tt[ok] - t_ends[ok]) < 1e-9)),
    }


def run_c3(args):
    line = batched_leg(args.solves, tile_config=args.tile_config, precision=64 if args.precision == "f64" and
                       args.c3_precision_given else 32, max_steps=args.c3_steps)
    line.update({"config_name": "c3", "n_gpus": 1, "data": "synthetic"})
    if os.environ.get("WENO_C3_ACCURACY", "1") != "0" and args.c3_steps is None:
        line["fp32_vs_fp64"] = batched_accuracy(args.solves)
    print(json.dumps(line))
    return 0


def run_c0(args):
    """The reference's own CPU-runnable case, end to end: 256^2 four-quadrant,
    component WENO5 (epsilon 1e-6) + HLLC (blend 1e4/1.1e4), CFL 0.5, 200 steps,
    FP64.  The same 200 steps are timed on the device solver (exact arithmetic,
    bit-identical to the oracle's run, and fast arithmetic; graph replay, state
    resident) and through host buffers (state in, 200 steps, state out), and on
    the host cores with the oracle."""
    import torch
    torch.cuda.set_device(0)
    import weno_ext
    from weno_ext import problems
    from oracle import oracle
    n, steps = 256, 200
    q0 = problems.quadrant(n, n, seed=20261200)
    kw = dict(cons=True, force_hlle=False, jp_cri=(1e4, 1.1e4), cfl=0.5, weno_eps=1e-6)
    runs = {}
    final = {}
    for mode in ("exact", "fast"):
        s = weno_ext.Solver(n, n, 1.0 / n, GAMMA, mode=mode, **kw)
        s.set_state(q0)
        s.run(steps)  # warm-up run (graph capture), then the timed one from the same state
        s.synchronize()
        s.set_state(q0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s.stream)
        s.run(steps)
        e1.record(s.stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        t0 = time.perf_counter()
        s.set_state(q0)
        s.run(steps)
        final[mode] = s.state()
        wall = time.perf_counter() - t0
        runs[f"fp64_{mode}"] = {"ms_per_step": ms / steps, "cell_updates_per_s": n * n * steps / (ms / 1e3),
                                "e2e_s": wall, "e2e_cell_updates_per_s": n * n * steps / wall,
                                "status": s.info()[2]}
        s.close()
    oracle.set_threads(0)
    oracle.set_weno_eps(1e-6)
    ref = q0.copy()
    t0 = time.perf_counter()
    try:
        for _ in range(steps):
            dt = 0.5 * (1.0 / n) / oracle.cfl_cmax(ref, n, n, GAMMA)
            oracle.rk3_step(ref, n, n, 1.0 / n, dt, GAMMA, False, (1e4, 1.1e4), True)
    finally:
        oracle.set_weno_eps(1e-12)
    cpu_s = time.perf_counter() - t0
    # one core (the reference's Rust core is single-threaded): the first 20 steps
    prev_threads = oracle.set_threads(0)
    oracle.set_threads(1)
    oracle.set_weno_eps(1e-6)
    r1 = q0.copy()
    t0 = time.perf_counter()
    try:
        for _ in range(20):
            dt = 0.5 * (1.0 / n) / oracle.cfl_cmax(r1, n, n, GAMMA)
            oracle.rk3_step(r1, n, n, 1.0 / n, dt, GAMMA, False, (1e4, 1.1e4), True)
    finally:
        oracle.set_weno_eps(1e-12)
        oracle.set_threads(prev_threads)
    one_s = (time.perf_counter() - t0) * steps / 20
    rel = {nm: v["rel_l1"] for nm, v in _l1_linf(final["fast"], ref).items()}
    line = {
        "metric": "200-step run of the 256^2 configuration (component WENO5 eps 1e-6 + HLLC, FP64)",
        "config_name": "c0", "value": runs["fp64_exact"]["e2e_cell_updates_per_s"], "unit": UNIT, "n_gpus": 1,
        "dtype": "f64", "data": "synthetic", "higher_is_better": True,
        "config": {"workload": "four-quadrant Riemann 256x256, cons-WENO5 (eps 1e-6) + GQ + HLLC, CFL 0.5, "
                               "200 steps", "seed": 20261200},
        "runs": runs,
        "exact_bit_identical_to_oracle": bool(np.array_equal(final["exact"], ref)),
        "fast_rel_l1_vs_oracle": rel,
        "cpu_oracle": {"seconds": cpu_s, "cell_updates_per_s": n * n * steps / cpu_s, "cores": os.cpu_count(),
                       "kind": "port"},
        "cpu_oracle_single_core": {"seconds_extrapolated": one_s, "cell_updates_per_s": n * n * steps / one_s,
                                   "cores": 1, "sample": "first 20 of the 200 steps, extrapolated"},
        "speedup_e2e_exact_vs_cpu": cpu_s / runs["fp64_exact"]["e2e_s"],
        "speedup_e2e_exact_vs_single_core": one_s / runs["fp64_exact"]["e2e_s"],
    }
    print(json.dumps(line))
    return 0


def run_dropin(args):
    """The reference-facing functions themselves (the weno_ext boundary) at nx x ny:
    l_local_py on torch CUDA tensors (device-resident) and on numpy arrays (host
    copies in and out every call), plus the per-direction sweeps it is built from.
    Unit: cell-residuals/s = interior cells whose L(U) one call evaluates, per second."""
    import torch
    torch.cuda.set_device(0)
    import weno_ext
    weno_ext.set_mode(args.mode)
    nx, ny = args.nx, args.ny
    q = quadrant_state(nx, ny)
    qd = torch.from_numpy(q).cuda()
    dx = 1.0 / nx
    k = max(args.steps, 1)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / k

    calls = {
        "l_local_py char+HLLE": lambda: weno_ext.l_local_py(qd, dx, GAMMA, True, (0.2, 1.0), False),
        "l_local_py char+blend": lambda: weno_ext.l_local_py(qd, dx, GAMMA, False, (0.2, 1.0), False),
        "l_local_py cons+HLLE": lambda: weno_ext.l_local_py(qd, dx, GAMMA, True, (0.2, 1.0), True),
        "weno_x_py": lambda: weno_ext.weno_x_py(qd, GAMMA),
        "weno_y_py": lambda: weno_ext.weno_y_py(qd, GAMMA),
        "flux_x_py": lambda: weno_ext.flux_x_py(qd, GAMMA),
        "con2primi_py": lambda: weno_ext.con2primi_py(qd, GAMMA),
    }
    ms = {name: timed(fn) for name, fn in calls.items()}
    ql, fl, qr, fr = weno_ext.weno_x_py(qd, GAMMA)
    ms["hlle_x_rs_py"] = timed(lambda: weno_ext.hlle_x_rs_py(ql, fl, qr, fr, GAMMA))
    ms["hllc_x_rs_py"] = timed(lambda: weno_ext.hllc_x_rs_py(ql, fl, qr, fr, GAMMA))
    del ql, fl, qr, fr
    # host arrays: the call copies the input in and the result out (the reference's calling convention)
    weno_ext.l_local_py(q, dx, GAMMA, True, (0.2, 1.0), False)
    t0 = time.perf_counter()
    for _ in range(k):
        weno_ext.l_local_py(q, dx, GAMMA, True, (0.2, 1.0), False)
    host_ms = (time.perf_counter() - t0) * 1e3 / k
    M, N = nx + 6, ny + 6
    main = ms["l_local_py char+HLLE"]
    alg = (M * N * 4 + nx * ny * 4) * 8  # stencil input once + residual out once
    peaks = load_json(os.path.join(ROOT, "MEASURED_PEAKS.json")) or {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    flops = (load_json(os.path.join(ROOT, "profiles", "flops_per_cell.json")) or {}).get("per_residual", {})
    fpc = flops.get("char_hlle", {}).get("flops")
    line = {
        "metric": "cell-residuals/s of l_local_py (char-WENO5+GQ+HLLE, FP64) on device tensors", "config_name": "dropin",
        "value": nx * ny / (main / 1e3), "unit": "cell-residuals/s", "n_gpus": 1, "dtype": "f64", "data": "synthetic",
        "higher_is_better": True, "mode": args.mode,
        "config": {"workload": f"four-quadrant Riemann {nx}x{ny} (+3 ghosts), one residual evaluation per call",
                   "nx": nx, "ny": ny, "calls_per_measurement": k},
        "ms_per_call": ms,
        "host_arrays": {"ms_per_call": host_ms, "value": nx * ny / (host_ms / 1e3), "unit": "cell-residuals/s",
                        "h2d_bytes": M * N * 8 * 8, "d2h_bytes": nx * ny * 4 * 8},
        "roofline": {"bound": "hbm", "achieved": alg / (main / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": alg / (main / 1e3) / 1e9 / hbm, "algorithmic_bytes": alg},
        "compute": ({"achieved_tflops": fpc * nx * ny / (main / 1e3) / 1e12, "flops_per_cell_residual": fpc}
                    if fpc else None),
    }
    print(json.dumps(line))
    return 0


def serving_leg(nreq, rate, lo, hi, t_end, budget_gb, fp64_fraction=0.25, slabs=4, max_wait_s=None, chunk_ms=25.0,
                accuracy_sample=8):
    """Serving: a seeded Poisson stream of requests (quadrant or oblique-shock initial
    data, FP32 or FP64 tag, seeded t_end) under an HBM budget with continuous batching."""
    import torch
    torch.cuda.set_device(0)
    from weno_ext import serving
    budget = int(budget_gb * 1e9)
    reqs = serving.poisson_stream(nreq, rate=rate, lo=lo, hi=hi, seed=SEED + 4, fp64_fraction=fp64_fraction,
                                  t_end=t_end, shock_fraction=0.3)
    # a seeded sample of FP32 requests keeps its result, to be compared with FP64 runs
    fp32 = [r.rid for r in reqs if r.precision == 32]
    sample = set(np.random.default_rng(SEED + 5).choice(fp32, size=min(accuracy_sample, len(fp32)),
                                                        replace=False).tolist()) if fp32 else set()
    srv = serving.Server(budget, slabs=slabs, max_solves=1024, steps_per_iter=8, max_wait_s=max_wait_s,
                         chunk_ms=chunk_ms, keep_results=sample)
    t0 = time.perf_counter()
    srv.serve(reqs, realtime=True)
    wall = time.perf_counter() - t0
    conversions = srv.conversions
    srv.close()
    summ = serving.summarize(reqs, wall)
    summ["slab_conversions"] = conversions
    if sample:
        # the same requests alone in FP64 (fast arithmetic, within 1e-10 of exact FP64)
        errs = []
        for r in reqs:
            if r.rid not in sample or r.status != 0:
                continue
            twin = serving.Request(**{k: getattr(r, k) for k in ("rid", "nx", "ny", "kind", "t_end", "seed", "mach",
                                                                  "theta")}, arrival=0.0, precision=64)
            solo = serving.Server(max(int(4e9), 4 * serving.footprint_bytes(r.nx, r.ny, 64) * 8), slabs=1,
                                  max_solves=2, keep_results=True)
            solo.serve([twin], realtime=False)
            solo.close()
            if twin.status == 0:
                a, b = r.result[3:-3, 3:-3, 0], twin.result[3:-3, 3:-3, 0]
                errs.append(float(np.abs(a - b).sum() / np.abs(b).sum()))
        if errs:
            summ["fp32_vs_fp64_rho_rel_l1"] = {"requests": len(errs), "median": float(np.median(errs)),
                                              "max": float(np.max(errs))}
    # work of each request (cells x steps) against its time to solution: the tail is
    # the largest requests, whose work spans more than three decades over [lo, hi]
    work = np.array([r.cells * r.steps for r in reqs if r.status == 0])
    tts = np.array([r.finished - r.arrival for r in reqs if r.status == 0])
    if len(work) > 2:
        summ["work_p50_over_p99"] = float(np.percentile(work, 50) / max(np.percentile(work, 99), 1))
        summ["corr_log_work_log_tts"] = float(np.corrcoef(np.log(work + 1), np.log(tts + 1e-9))[0, 1])
    return {"metric": "p50/p99 time-to-solution and aggregate cell-updates/s, serving stream",
            "value": summ["aggregate_cell_updates_per_s"], "unit": UNIT, "dtype": "f32+f64",
            "config": {"workload": f"{nreq} Poisson requests at {rate}/s, edges log-uniform [{lo},{hi}], "
                                   f"t_end~U{tuple(t_end)}, {int(100 * fp64_fraction)}% FP64, 30% oblique shock, "
                                   f"HBM budget {budget / 1e9:.0f} GB in {slabs} slabs",
                       "first_chunk_steps": 8, "chunk_ms": chunk_ms, "max_wait_s": max_wait_s},
            "serving": summ}


def run_c4(args):
    lo, hi = int(os.environ.get("WENO_C4_LO", "128")), int(os.environ.get("WENO_C4_HI", "2048"))
    rate = float(os.environ.get("WENO_C4_RATE", "10"))
    t_end = (float(os.environ.get("WENO_C4_TLO", "0.001")), float(os.environ.get("WENO_C4_THI", "0.003")))
    budget = float(os.environ.get("WENO_C4_BUDGET_GB", "150"))
    wait = os.environ.get("WENO_C4_MAX_WAIT")
    line = serving_leg(args.requests, rate, lo, hi, t_end, budget, max_wait_s=float(wait) if wait else None,
                       chunk_ms=float(os.environ.get("WENO_C4_CHUNK_MS", "25")))
    line.update({"config_name": "c4", "n_gpus": 1, "data": "synthetic"})
    print(json.dumps(line))
    return 0


def dropin_host_leg(nx, ny, calls=3):
    """The reference's calling convention: l_local_py on numpy arrays of the drivers'
    (nx+6, ny+6, 8) layout, host copies in and out inside every call, both arithmetic
    modes.  Unit: cell-residuals/s (interior cells whose L(U) one call evaluates)."""
    import weno_ext
    q = quadrant_state(nx, ny)
    dx = 1.0 / nx
    out = {}
    prev = weno_ext.get_mode()
    try:
        for mode in ("fast", "exact"):
            weno_ext.set_mode(mode)
            weno_ext.l_local_py(q, dx, GAMMA, True, (0.2, 1.0), False)
            t0 = time.perf_counter()
            for _ in range(calls):
                weno_ext.l_local_py(q, dx, GAMMA, True, (0.2, 1.0), False)
            ms = (time.perf_counter() - t0) * 1e3 / calls
            out[mode] = {"ms_per_call": ms, "value": nx * ny / (ms / 1e3)}
    finally:
        weno_ext.set_mode(prev)
    M, N = nx + 6, ny + 6
    return {"value": out["fast"]["value"], "unit": "cell-residuals/s", "modes": out,
            "h2d_bytes_per_call": M * N * 8 * 8, "d2h_bytes_per_call": nx * ny * 4 * 8,
            "path": "weno_ext.l_local_py(numpy (nx+6, ny+6, 8) f64, dx, 1.4, True, (0.2, 1.0), False) -> numpy "
                    "(nx, ny, 4); char-WENO5+GQ+HLLE, one residual per call",
            "calls": calls}


def time_solver(Solver, q0, nx, ny, steps, warmup, **kw):
    """Device-resident run; returns (ms for `steps` timed steps, solver)."""
    import torch
    s = Solver(nx, ny, 1.0 / nx, GAMMA, **kw)
    s.set_state(q0)
    s.run(warmup, graph=True)
    s.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s.stream)
    s.run(steps, graph=True)
    e1.record(s.stream)
    e1.synchronize()
    return e0.elapsed_time(e1), s


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=4096)
    ap.add_argument("--ny", type=int, default=4096)
    ap.add_argument("--mode", default="fast", choices=["fast", "exact"])
    ap.add_argument("--precision", default="f64", choices=["f64", "df64", "f32"],
                    help="arithmetic of the headline solver (f64 = IEEE double, the default; df64 = double-float "
                         "pairs on the FP32 pipes; f32)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--config", default="headline", choices=["headline", "c0", "c1", "c2", "c3", "c4", "dropin"],
                    help="headline: the 4096^2 FP64 step (default); c0: the 256^2 200-step run end to end; "
                         "c1: 2048^2 FP64/FP32 accuracy run; "
                         "c2: oblique shock 4096x1024 FP32 vs FP64; c3: batched uneven solves; c4: serving stream; "
                         "dropin: the weno_ext functions themselves (l_local_py & co.)")
    ap.add_argument("--solves", type=int, default=512)
    ap.add_argument("--c3-steps", type=int, default=None,
                    help="c3: cap every solve at this many steps (short runs for profiling)")
    ap.add_argument("--tile-config", type=int, default=None,
                    help="c3: run the batch with this tile configuration instead of the autotuned one "
                         "(0-3 fused tile kernel, 4 staged kernels)")
    ap.add_argument("--requests", type=int, default=300)
    ap.add_argument("--no-batched", action="store_true", help="skip the batched (512 solves) leg of the default line")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream leg of the default line")
    ap.add_argument("--no-dropin", action="store_true", help="skip the numpy l_local_py leg of the default line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    # c3 is the FP32 configuration; --precision f64 given explicitly runs the same batch in FP64
    args.c3_precision_given = any(a == "--precision" or a.startswith("--precision=") for a in sys.argv[1:])
    if args.impl == "reference":
        return run_reference(args)
    if args.config in ("c1", "c2"):
        return run_accuracy(args)
    if args.config == "c3":
        return run_c3(args)
    if args.config == "c4":
        return run_c4(args)
    if args.config == "dropin":
        return run_dropin(args)
    if args.config == "c0":
        return run_c0(args)

    import torch
    from weno_ext import replicas
    world, rank, local = replicas.world()
    torch.cuda.set_device(local if world > 1 else 0)
    replicas.init("nccl")
    import weno_ext
    from weno_ext import _lib
    L = _lib.load()

    nx, ny = args.nx, args.ny
    q0 = quadrant_state(nx, ny)
    prec_code = {"f64": 64, "df64": 48, "f32": 32}[args.precision]
    kw = dict(precision=prec_code, mode=args.mode, cons=False, force_hlle=True, jp_cri=(0.2, 1.0), cfl=0.45)
    s = weno_ext.Solver(nx, ny, 1.0 / nx, GAMMA, **kw)
    s.set_state(q0)
    s.run(args.warmup, graph=False)
    s.synchronize()

    # ---- timed region: K steps, per-kernel-class events on the solver stream ----
    import ctypes
    _lib.check(L.weno_solver_enable_timing(s._h, 1), "timing")
    clocks = ClockSampler(torch.cuda.current_device())
    replicas.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s.stream)
    s.run(args.steps, graph=False)
    e1.record(s.stream)
    e1.synchronize()
    torch.cuda.synchronize()
    replicas.barrier()
    clk = clocks.stop()
    ms = replicas.max_over_ranks(e0.elapsed_time(e1), device="cuda")
    ms_cls = (ctypes.c_double * len(CLASSES))()
    n_cls = (ctypes.c_int64 * len(CLASSES))()
    _lib.check(L.weno_solver_timing_report(s._h, ms_cls, n_cls, len(CLASSES)), "timing report")
    _lib.check(L.weno_solver_enable_timing(s._h, 0), "timing")
    t_sim, nsteps_done, status = s.info()
    launches = s.launches_per_step * args.steps
    value = replicas.job_rate(nx * ny * args.steps, ms, world)

    # ---- dominant kernel and its roofline ----
    kern = {CLASSES[i]: {"ms": ms_cls[i], "launches": int(n_cls[i])} for i in range(len(CLASSES)) if n_cls[i]}
    dom = max(kern, key=lambda k: kern[k]["ms"])
    M, N = nx + 6, ny + 6
    es = 4 if args.precision == "f32" else 8
    # Algorithmic bytes per launch: the stencil input once plus the outputs once.
    alg_bytes = {
        "pass1_x": (4 * M * N + 8 * (M - 5) * N) * es,
        "pass1_y": (4 * M * N + 8 * M * (N - 5)) * es,
        "pass2_x": (8 * (M - 5) * N + 4 * (M - 5) * (N - 6)) * es,
        "pass2_y": (8 * M * (N - 5) + 4 * (M - 6) * (N - 5)) * es,
        "residual+rk": (8 * (M - 5) * (N - 6) // 2 + 4 * (M - 6) * (N - 5) + 12 * nx * ny) * es,
    }
    peaks = load_json(os.path.join(ROOT, "MEASURED_PEAKS.json")) or {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    per_launch_ms = kern[dom]["ms"] / max(kern[dom]["launches"], 1)
    achieved = alg_bytes.get(dom, 0) / (per_launch_ms / 1e3) / 1e9 if dom in alg_bytes else None
    prof = load_json(os.path.join(ROOT, "profiles", "roofline_traffic.json")) or {}
    traffic = prof.get(dom, {}).get("dram_bytes_per_launch") if isinstance(prof.get(dom), dict) else None
    if args.precision != "f64":
        traffic = None  # the committed DRAM capture is of the FP64 kernels
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if achieved else None, "traffic": traffic,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"}
    # The whole step against the minimal fused traffic of one cell-update: 32 values
    # (stage 1 reads 4, writes 4; stages 2 and 3 read 8, write 4), 256 B in FP64.
    step_bytes = 32 * (4 if args.precision == "f32" else 8) * nx * ny
    step_gbs = step_bytes / (ms / args.steps / 1e3) / 1e9
    roofline["step"] = {"algorithmic_bytes_per_step": step_bytes, "achieved": step_gbs, "unit": "GB/s",
                        "frac": step_gbs / hbm_peak,
                        "note": "32 values per cell-update (minimal fused SSP-RK3 traffic) x cells / ms_per_step"}
    roofline["step_frac_8d"] = step_gbs / hbm_peak
    pipe = prof.get("fp64_pipe_pct_of_peak") if args.precision == "f64" else None
    if pipe:
        # The HBM fraction is the contract's denominator; the pipe that binds these kernels is FP64.
        roofline["binding"] = {"pipe": "fp64", "ncu_fp64_pipe_pct": pipe,
                               "source": "profiles/k_pass1_k_pass2_fp64_fast_2048.md (ncu, 2048^2)"}
    r64, rdiv, r32 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _lib.check(L.weno_probe_rates(ctypes.byref(r64), ctypes.byref(rdiv), ctypes.byref(r32), None), "probe")
    flops = load_json(os.path.join(ROOT, "profiles", "flops_per_cell.json")) or {}
    fpc = flops.get("char_hlle_step")
    compute = None
    if fpc and r64.value > 0 and args.precision == "f64":
        ach = fpc * value / world / 1e12
        compute = {"bound": "fp64", "achieved": ach, "peak": r64.value, "unit": "TFLOP/s",
                   "frac": ach / r64.value, "flops_per_cell_update": fpc,
                   "measured_rates": {"fp64_fma_tflops": r64.value, "fp64_div_per_s": rdiv.value,
                                      "fp32_fma_tflops": r32.value},
                   "note": "algorithmic FLOPs of the reference algorithm per cell-update (oracle tally: add, mul, "
                           "div and sqrt count 1 each); peak = FP64 FMA rate measured live on this GPU"}

    # ---- e2e: public API with host buffers, H2D + D2H every step ----
    host = torch.empty((M, N, 8), dtype=torch.float64).pin_memory()
    host.numpy()[:] = q0
    hp = host.data_ptr()
    s2 = weno_ext.Solver(nx, ny, 1.0 / nx, GAMMA, **kw)
    L.weno_solver_set_state_host(s2._h, hp, 8)
    s2.run(1, graph=True)
    L.weno_solver_get_state_host(s2._h, hp)
    torch.cuda.synchronize()
    clocks_e2e = ClockSampler(torch.cuda.current_device())
    clocks_e2e.start()
    pc = time.perf_counter
    split = np.zeros(3)
    t0 = pc()
    evs = []
    for _ in range(args.e2e_steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ta = pc()
        _lib.check(L.weno_solver_set_state_host(s2._h, hp, 8), "e2e set_state")  # returns after the upload
        tb = pc()
        ev[0].record(s2.stream)
        s2.run(1, graph=True)
        ev[1].record(s2.stream)
        _lib.check(L.weno_solver_get_state_host(s2._h, hp), "e2e get_state")  # waits for the step and the download
        ev[2].record(s2.stream)
        tc = pc()
        split += (tb - ta, tc - tb, tc - ta)
        evs.append(ev)
    torch.cuda.synchronize()
    e2e_s = pc() - t0
    dev_step = sum(ev[0].elapsed_time(ev[1]) for ev in evs) / len(evs)
    clk_e2e = clocks_e2e.stop()
    e2e = {"value": nx * ny * args.e2e_steps * world / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": M * N * 8 * 8, "d2h_bytes_per_step": M * N * 8 * 8,
           "ms_per_step": 1e3 * e2e_s / args.e2e_steps,
           "ms_upload": 1e3 * split[0] / args.e2e_steps, "ms_step_and_download": 1e3 * split[1] / args.e2e_steps,
           "ms_device_step": dev_step, "clocks": clk_e2e,
           "path": "weno_solver_set_state_host -> run(1) -> weno_solver_get_state_host, pinned host buffer"}
    s2.close()

    # ---- other variants (timed separately, graph replay) ----
    variants = {}
    if not args.no_variants:
        for name, vkw, k in (("fp64_exact", dict(kw, mode="exact"), max(2, args.steps // 3)),
                             ("fp32", dict(kw, precision=32, mode="fast"), args.steps * 4),
                             ("df64", dict(kw, precision=48, mode="fast"), args.steps * 2),
                             ("fp64_fast_hllc_blend", dict(kw, force_hlle=False, jp_cri=(1e4, 1.1e4)),
                              max(2, args.steps // 2))):
            vms, vs = time_solver(weno_ext.Solver, q0, nx, ny, k, 3, **vkw)
            variants[name] = {"value": nx * ny * k / (vms / 1e3), "unit": UNIT, "steps": k, "ms_per_step": vms / k}
            vs.close()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
        "config": {"workload": f"four-quadrant Riemann {nx}x{ny}, char-WENO5 + 2-pt Gauss faces + HLLE, "
                               f"SSP-RK3, CFL 0.45, {args.precision} ({args.mode} arithmetic)",
                   "nx": nx, "ny": ny, "seed": SEED, "mode": args.mode,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (state 4 x (nx+6)(ny+6) f64 = %.0f MB per buffer)" %
                         (4 * M * N * 8 / 1e6)},
        "roofline": roofline,
        "compute_roofline": compute,
        "kernels_ms": kern,
        "clocks": clk,
        "gpu_launches": launches,
        "e2e": e2e,
        "variants": variants,
        "status": {"sim_time": t_sim, "steps_done": nsteps_done, "numeric_status": status},
    }
    line["parity"] = {
        "exact_vs_oracle": "bit-identical after 2 steps of this workload at 4096^2 "
                           "(tests/test_gpu_headline.py)",
        "fast_vs_exact": "relative L1 <= 1e-10 per conserved variable after 25 steps of this workload "
                         "(tests/test_gpu_headline.py; measured 3.3e-16)"}
    s.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(nx, int(os.environ.get("WENO_CPU_STRIP", "32")), os.cpu_count() or 1)
    if rank == 0 and world == 1 and args.precision == "f64" and (nx, ny) == (4096, 4096):
        # The headline metric's other figures (the drop-in call rate, the batched FP32
        # rate, the serving p50/p99), on the same box in the same run (the default
        # workload only: smaller --nx/--ny runs are profiling cases).
        torch.cuda.empty_cache()
        if not args.no_dropin:
            line["e2e_dropin"] = dropin_host_leg(nx, ny)
        if not args.no_batched:
            line["batched"] = batched_leg(args.solves)
        if not args.no_serving:
            line["serving"] = serving_leg(int(os.environ.get("WENO_SERVE_REQUESTS", "200")), 20.0, 128, 2048,
                                          (0.001, 0.003), 150.0)
    if rank == 0:
        print(json.dumps(line))
    replicas.finish()
    return 0


if __name__ == "__main__":
    sys.exit(main())
