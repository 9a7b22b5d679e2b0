"""Record the reference drivers' own calls into weno_ext, for the driver replay test.

Usage (a checkout of the reference is needed; nothing here reads it by default):

    WENO_REFERENCE_DIR=<reference checkout> python tests/golden/make_driver_trace.py

The reference drivers ``Rie_prob_2d_rs.main_rs`` (rk3_cc, _sync_primitives,
apply_bc_zero_gradient, apply_bc_reflecting; Rie_prob_2d_rs.py:123-207,213-365)
and ``double_mach_reflection.main_rs`` (rk3_refac with its five-argument
l_local_py calls and con2primi_py; double_mach_reflection.py:97-134,176-300,
unitest.py:169-227) are imported unchanged and run end to end with a stand-in
``weno_ext`` module that records every call: the function, the call form (how
many positional arguments, which keywords), the scalar arguments, and a
SHA-256 digest of every array going in and coming out.  The stand-in computes
with the oracle (the C++ restatement of the Rust core); for the
component-wise + HLLE run the same trace is recorded a second time with the
reference's own numpy twin (WENO_HLLC_2d.py) as the backend and the two traces
must agree digest for digest, which pins that chain to the reference's Python.

Written to tests/golden/driver_trace.npz: per run, the first input of the run
(the driver's initial array after its boundary fill; compressed, piecewise
constant), the trace as JSON, and the digest of the array main_rs returns.
The replay test (tests/test_gpu_driver_replay.py) re-enacts the same calls on
the product package and checks every digest, so that a run of the unchanged
driver on this package is shown to produce the same arrays, call by call.
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
GAMMA = 1.4
RUST_SQRT3_12 = 0.1443375673


def digest(a) -> str:
    """SHA-256 over shape and C-order float64 bytes, every NaN replaced by one bit pattern
    (NaN payloads differ between CPU architectures and the GPU)."""
    if isinstance(a, tuple):
        return hashlib.sha256("".join(digest(x) for x in a).encode()).hexdigest()
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    a = np.where(np.isnan(a), np.nan, a)
    h = hashlib.sha256(repr(a.shape).encode())
    h.update(a.tobytes())
    return h.hexdigest()


def _reference_dir():
    ref = os.environ.get("WENO_REFERENCE_DIR")
    if not ref or not os.path.isdir(ref):
        sys.exit("set WENO_REFERENCE_DIR to a checkout of the reference (colinhu123/WENO-CFD-solver)")
    return ref


def _install_stubs():
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    for name in ("figure", "imshow", "show", "plot", "colorbar", "title", "close", "subplots", "pause"):
        setattr(plt, name, lambda *a, **k: None)
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt
    pu = types.ModuleType("plot_utils")
    pu.interactive_plot_keyboard = lambda *a, **k: None
    sys.modules["plot_utils"] = pu


class Recorder:
    """A weno_ext stand-in: the twelve names of the reference module, each computed by
    `backend` and logged."""

    NAMES = ("flux_x_py", "flux_y_py", "con2primi_py", "weno_x_py", "weno_y_py", "hllc_x_rs_py", "hllc_y_rs_py",
             "hlle_x_rs_py", "hlle_y_rs_py", "hllc_hlle_x_rs_py", "hllc_hlle_y_rs_py", "l_local_py")

    def __init__(self, backend):
        self.calls = []
        self.first_input = None
        self.module = types.ModuleType("weno_ext")
        for name in self.NAMES:
            if hasattr(backend, name):
                setattr(self.module, name, self._wrap(name, getattr(backend, name)))

    def _wrap(self, name, fn):
        def call(*args, **kwargs):
            out = fn(*args, **kwargs)
            arrays = [a for a in list(args) + list(kwargs.values()) if isinstance(a, np.ndarray)]
            if self.first_input is None:
                self.first_input = np.array(arrays[0], copy=True)
            scalars = {}
            for k, a in enumerate(args):
                if not isinstance(a, np.ndarray):
                    scalars[str(k)] = list(a) if isinstance(a, tuple) else a
            for k, a in kwargs.items():
                if not isinstance(a, np.ndarray):
                    scalars[k] = list(a) if isinstance(a, tuple) else a
            self.calls.append({"fn": name, "npos": len(args), "kw": sorted(kwargs), "scalars": scalars,
                               "in": [digest(a) for a in arrays],
                               "out": digest(tuple(out) if isinstance(out, (tuple, list)) else out)})
            return out
        return call


class OracleBackend:
    """The oracle's functions under the reference module's signatures (cons_switch
    defaults to False, the characteristic reconstruction, as in lib.rs)."""

    def __init__(self):
        sys.path.insert(0, ROOT)
        from oracle import oracle
        oracle.build()
        oracle.set_threads(0)
        self.o = oracle

    def l_local_py(self, u, dx, gamma, force_hlle, jp_cri, cons_switch=False):
        return self.o.l_local_py(u, dx, gamma, force_hlle, jp_cri, cons_switch)

    def con2primi_py(self, q, gamma):
        return self.o.con2primi_py(q, gamma)


class TwinBackend:
    """The reference's numpy twin (component-wise + HLLE only), with the Rust core's
    SQRT3_12 literal; con2primi's sixth output is the enthalpy the Rust core returns."""

    def __init__(self, twin):
        self.twin = twin

    def l_local_py(self, u, dx, gamma, force_hlle, jp_cri, cons_switch=False):
        if not (force_hlle and cons_switch):
            raise RuntimeError("the numpy twin covers only the component-wise + HLLE configuration")
        return self.twin.L(u, dx, gamma, True, jp_cri)

    def con2primi_py(self, q, gamma):
        p, a, rho, u, v = self.twin.con2primi(q, gamma)
        return p, a, rho, u, v, (q[:, :, 3] + p) / rho


def _fresh_import(ref, stand_in):
    for mod in ("weno_ext", "Rie_prob_2d_rs", "double_mach_reflection", "unitest"):
        sys.modules.pop(mod, None)
    sys.modules["weno_ext"] = stand_in
    if ref not in sys.path:
        sys.path.insert(0, ref)
    import Rie_prob_2d_rs as rie  # noqa: E402
    import double_mach_reflection as dmr  # noqa: E402
    return rie, dmr


RIE_GRID = {"nx": 64, "ny": 64, "dx": 1 / 64}
DMR_GRID = {"nx": 128, "ny": 32, "dx": 1 / 32, "x": 4, "y": 1}
RUNS = {
    # Rie_prob_2d_rs.main_rs, step-controlled (10 steps): the reference init (quadrants
    # split at 0.75 nx, reflecting fill), then rk3_cc with six-argument l_local_py calls.
    "rie_cons_hlle": ("rie", RIE_GRID, {"nstep": 10, "CFL": 0.45, "force_hlle": True, "jp_cri": (0.2, 1.0),
                                        "weno type": True}),
    "rie_char_hlle": ("rie", RIE_GRID, {"nstep": 10, "CFL": 0.45, "force_hlle": True, "jp_cri": (0.2, 1.0),
                                        "weno type": False}),
    "rie_char_blend": ("rie", RIE_GRID, {"nstep": 10, "CFL": 0.45, "force_hlle": False, "jp_cri": (0.05, 0.4),
                                         "weno type": False}),
    # double_mach_reflection.main_rs, time-controlled with a 10-step cap: unitest.init_refac,
    # rk3_refac with five-argument l_local_py calls (cons_switch left at its default).
    "dmr_char_hllc": ("dmr", DMR_GRID, {"nstep": 10, "t_final": 0.2, "CFL": 0.1, "force_hlle": False,
                                        "jp_cri": (10000, 11000)}),
}


def record(ref, backend, run):
    kind, grid, ctrl = RUNS[run]
    rec = Recorder(backend)
    rie, dmr = _fresh_import(ref, rec.module)
    ctrl = dict(ctrl, file_storage=False, visualize=False, mode="opt")
    driver = rie if kind == "rie" else dmr
    q = driver.main_rs(dict(grid), ctrl, {"gamma": GAMMA})
    return rec, q


def main():
    ref = _reference_dir()
    _install_stubs()
    orc = OracleBackend()
    out, meta = {}, {}
    for run, (kind, grid, ctrl) in RUNS.items():
        rec, q = record(ref, orc, run)
        finite = bool(np.isfinite(q[:, :, :4]).all())
        meta[run] = {"driver": kind, "grid": grid, "control": {k: (list(v) if isinstance(v, tuple) else v)
                                                                 for k, v in ctrl.items()},
                     "calls": rec.calls, "final": digest(q), "finite": finite, "backend": "oracle"}
        out[f"{run}/first_input"] = rec.first_input
        print(run, len(rec.calls), "calls, final finite:", finite)
    # The component-wise + HLLE chain once more on the reference's own numpy twin.
    sys.path.insert(0, ref)
    import WENO_HLLC_2d as twin  # noqa: E402
    twin.SQRT3_12 = RUST_SQRT3_12
    rec, q = record(ref, TwinBackend(twin), "rie_cons_hlle")
    same = [a["out"] == b["out"] and a["in"] == b["in"] for a, b in zip(rec.calls, meta["rie_cons_hlle"]["calls"])]
    if not (all(same) and len(same) == len(rec.calls) and digest(q) == meta["rie_cons_hlle"]["final"]):
        sys.exit("oracle and numpy-twin traces of the component-wise + HLLE run differ")
    meta["rie_cons_hlle"]["backend"] = "oracle, identical to the reference's numpy twin (WENO_HLLC_2d.py)"
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "driver_trace.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
