"""Generate the golden vectors that pin the CPU oracle to the reference.

Run with the path of a checkout of the reference sources in WENO_REFERENCE_DIR
(there is no default location):

    WENO_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py

The reference's Rust extension cannot be built here (no Rust toolchain), so the
vectors come from the reference's own Python code, imported unchanged:

* ``WENO_HLLC_2d.py`` -- the numpy twin of the component-wise reconstruction,
  the HLLE solver, con2primi, the flux functions, the pressure-gradient sensor
  and the residual ``L``.  Its module constant ``SQRT3_12`` is np.sqrt(3)/12,
  while the Rust core uses the literal 0.1443375673 (weno_ext/src/utils.rs:4);
  the twin is run with the constant set to the Rust literal so that it
  computes what the Rust core computes.  Its HLLC differs from the Rust one in
  the star-right branch (WENO_HLLC_2d.py:476 vs riemann.rs:67), so HLLC faces
  are stored with a mask of the faces whose star speed is clearly >= 0.
* ``Rie_prob_2d_rs.py``, ``double_mach_reflection.py`` and ``unitest.py`` --
  the drivers (initial data, boundary fills, SSP-RK3, CFL), run end to end with
  a stand-in ``weno_ext`` module backed by the numpy twin, which requires the
  component-wise + HLLE configuration.

matplotlib, plot_utils and weno_ext are replaced by stub modules before import;
no reference file is modified.  Outputs: tests/golden/*.npz (small).
"""

from __future__ import annotations

import os
import sys
import types

import numpy as np

REF = os.environ.get("WENO_REFERENCE_DIR", "")
OUT = os.path.dirname(os.path.abspath(__file__))
RUST_SQRT3_12 = 0.1443375673
GAMMA = 1.4


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


def _import_reference():
    if not REF or not os.path.isdir(REF):
        sys.exit("set WENO_REFERENCE_DIR to a checkout of the reference (colinhu123/WENO-CFD-solver)")
    _install_stubs()
    sys.path.insert(0, REF)
    import WENO_HLLC_2d as twin  # noqa: E402
    twin.SQRT3_12 = RUST_SQRT3_12

    # Stand-in weno_ext backed by the numpy twin (component-wise + HLLE only).
    we = types.ModuleType("weno_ext")

    def l_local_py(u, dx, gamma, force_hlle, jp_cri, cons_switch=True):
        if not (force_hlle and cons_switch):
            raise RuntimeError("the numpy twin covers only the component-wise + HLLE configuration")
        return twin.L(u, dx, gamma, True, jp_cri)

    def con2primi_py(q, gamma):
        p, a, rho, u, v = twin.con2primi(q, gamma)
        h = (q[:, :, 3] + p) / rho
        return p, a, rho, u, v, h

    we.l_local_py = l_local_py
    we.con2primi_py = con2primi_py
    sys.modules["weno_ext"] = we
    import Rie_prob_2d_rs as rie  # noqa: E402
    import unitest  # noqa: E402
    import double_mach_reflection as dmr  # noqa: E402
    return twin, rie, unitest, dmr


def quadrant_state(rng, nx, ny, split=0.5, gamma=GAMMA, channels=8):
    """Four-quadrant state: per-quadrant rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]."""
    q = np.zeros((nx + 6, ny + 6, channels))
    si = 3 + int(split * nx)
    sj = 3 + int(split * ny)
    for qi, (a, b) in enumerate([(slice(None, si), slice(None, sj)), (slice(si, None), slice(None, sj)),
                                 (slice(None, si), slice(sj, None)), (slice(si, None), slice(sj, None))]):
        rho, p = rng.uniform(0.1, 2.0, 2)
        u, v = rng.uniform(-1.0, 1.0, 2)
        q[a, b, 0] = rho
        q[a, b, 1] = rho * u
        q[a, b, 2] = rho * v
        q[a, b, 3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return q


def smooth_state(rng, m, n, channels=8, gamma=GAMMA):
    x = np.linspace(0, 1, m)[:, None]
    y = np.linspace(0, 1, n)[None, :]
    k = rng.uniform(1, 4, 4)
    rho = 1.0 + 0.3 * np.sin(2 * np.pi * k[0] * x + 1.3 * y)
    u = 0.5 * np.cos(2 * np.pi * k[1] * y + x)
    v = 0.4 * np.sin(2 * np.pi * k[2] * (x + y))
    p = 1.0 + 0.2 * np.cos(2 * np.pi * k[3] * x * y)
    q = np.zeros((m, n, channels))
    q[:, :, 0] = rho
    q[:, :, 1] = rho * u
    q[:, :, 2] = rho * v
    q[:, :, 3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return q


def star_speed_mask(qL, qR, gamma, ydir):
    """Faces whose HLLC star speed is clearly non-negative (|S*| > 1e-6).

    Written independently of the twin: Roe-averaged speeds and Toro's S*.
    """
    eps = 1e-12
    rl = np.maximum(qL[..., 0], eps)
    rr = np.maximum(qR[..., 0], eps)
    ul, vl = qL[..., 1] / rl, qL[..., 2] / rl
    ur, vr = qR[..., 1] / rr, qR[..., 2] / rr
    pl = np.maximum((gamma - 1) * (qL[..., 3] - 0.5 * rl * (ul ** 2 + vl ** 2)), eps)
    pr = np.maximum((gamma - 1) * (qR[..., 3] - 0.5 * rr * (ur ** 2 + vr ** 2)), eps)
    hl, hr = (qL[..., 3] + pl) / rl, (qR[..., 3] + pr) / rr
    sl_, sr_ = np.sqrt(rl), np.sqrt(rr)
    ut = (sl_ * ul + sr_ * ur) / (sl_ + sr_)
    vt = (sl_ * vl + sr_ * vr) / (sl_ + sr_)
    ht = (sl_ * hl + sr_ * hr) / (sl_ + sr_)
    at = np.sqrt(np.maximum((gamma - 1) * (ht - 0.5 * (ut ** 2 + vt ** 2)), 0))
    unl, unr, unt = (vl, vr, vt) if ydir else (ul, ur, ut)
    SL, SR = unt - at, unt + at
    den = rl * (SL - unl) - rr * (SR - unr)
    Ss = (pr - pl + rl * unl * (SL - unl) - rr * unr * (SR - unr)) / den
    return (Ss > 1e-6) | (SL > 1e-6)


def make_twin(twin):
    rng = np.random.default_rng(20260101)
    cases = {}
    cases["quad"] = quadrant_state(rng, 14, 11)
    cases["smooth"] = smooth_state(rng, 19, 17)
    q = quadrant_state(rng, 12, 12)
    q[:, :, 4:] = rng.uniform(-5, 5, q[:, :, 4:].shape)  # primitive channels are never read
    cases["quad8"] = q
    out = {}
    for name, u in cases.items():
        out[f"{name}/u"] = u
        qLx, FLx, qRx, FRx = twin.weno_x(u, GAMMA)
        qLy, FLy, qRy, FRy = twin.weno_y(u, GAMMA)
        for tag, arr in (("qlx", qLx), ("flx", FLx), ("qrx", qRx), ("frx", FRx),
                         ("qly", qLy), ("fly", FLy), ("qry", qRy), ("fry", FRy)):
            out[f"{name}/{tag}"] = arr
        out[f"{name}/flux_x"] = twin.flux_x(u[:, :, :4], GAMMA)
        out[f"{name}/flux_y"] = twin.flux_y(u[:, :, :4], GAMMA)
        p, a, rho, uu, vv = twin.con2primi(u, GAMMA)
        for tag, arr in (("p", p), ("a", a), ("rho", rho), ("uu", uu), ("vv", vv)):
            out[f"{name}/c2p_{tag}"] = arr
        out[f"{name}/hlle_x"] = twin.HLLE_x(qLx, qRx, FLx, FRx, GAMMA)
        out[f"{name}/hlle_y"] = twin.HLLE_y(qLy, qRy, FLy, FRy, GAMMA)
        out[f"{name}/hllc_x"] = twin.HLLC_x(qLx, qRx, FLx, FRx, GAMMA)
        out[f"{name}/hllc_y"] = twin.HLLC_y(qLy, qRy, FLy, FRy, GAMMA)
        out[f"{name}/hllc_x_mask"] = star_speed_mask(qLx, qRx, GAMMA, False)
        out[f"{name}/hllc_y_mask"] = star_speed_mask(qLy, qRy, GAMMA, True)
        pl = twin.con2primi(qLx, GAMMA)[0]
        pr = twin.con2primi(qRx, GAMMA)[0]
        out[f"{name}/sensor_x"] = twin.shock_sensor_grad_p(pr, pl, 0.05, 0.4)
        out[f"{name}/sensor_pbar_x"] = 0.5 * (pl + pr)
        dx = 1.0 / max(u.shape[0] - 6, 1)
        out[f"{name}/dx"] = np.array(dx)
        out[f"{name}/L_hlle"] = twin.L(u, dx, GAMMA, True, (0.2, 1.0))
    np.savez_compressed(os.path.join(OUT, "twin_cons_hlle.npz"), **out)


def make_drivers(rie, unitest, dmr):
    out = {}
    # Rie_prob_2d_rs: reference init (quadrant split at 0.75*nx) and main_rs in
    # step-controlled and time-controlled mode, "mode": "opt" returns q.
    grid = {"nx": 16, "ny": 16, "dx": 1 / 16}
    ctrl = {"nstep": 3, "CFL": 0.3, "file_storage": False, "force_hlle": True, "visualize": False,
            "mode": "opt", "jp_cri": (0.5, 2), "weno type": True}
    out["rie/q0"] = rie.init(grid, ctrl, GAMMA)
    out["rie/q_nstep3"] = rie.main_rs(grid, dict(ctrl), {"gamma": GAMMA})
    ctrl_t = dict(ctrl, t_final=0.02, nstep=50)
    out["rie/q_tfinal"] = rie.main_rs(grid, ctrl_t, {"gamma": GAMMA})
    out["rie/t_final"] = np.array(0.02)
    # One rk3_cc step on a seeded random quadrant state with a fixed dt.
    rng = np.random.default_rng(7)
    q = quadrant_state(rng, 13, 10)
    q = rie.apply_bc_zero_gradient(q, None)
    rie._sync_primitives(q, GAMMA)
    out["rk3/q_in"] = q.copy()
    out["rk3/q_out"] = rie.rk3_cc(q.copy(), {"nx": 13, "ny": 10, "dx": 0.05}, 1e-3, GAMMA, True, True, (0.2, 1.0))
    # double_mach_reflection: unitest.init_refac + main_rs (t_final mode) on a small grid.
    dgrid = {"nx": 40, "ny": 10, "dx": 1 / 10, "x": 4, "y": 1}
    dctrl = {"nstep": 4, "CFL": 0.1, "file_storage": False, "force_hlle": True, "visualize": False,
             "mode": "opt", "t_final": 0.01, "jp_cri": (10000, 11000)}
    q0, bound = unitest.init_refac(dgrid, dctrl, GAMMA)
    out["dmr/q0"] = q0
    out["dmr/bound"] = np.array(bound)
    out["dmr/q_final"] = dmr.main_rs(dgrid, dctrl, {"gamma": GAMMA})
    # Boundary fills on random arrays (every ghost cell starts as noise).
    rng = np.random.default_rng(11)
    a = rng.standard_normal((19, 15, 8))
    out["bc/rand"] = a
    out["bc/zero_gradient"] = rie.apply_bc_zero_gradient(a.copy(), None)
    sq = rng.standard_normal((17, 17, 8))
    out["bc/rand_sq"] = sq
    out["bc/reflecting"] = rie.apply_bc_reflecting(sq.copy(), None)
    b = rng.standard_normal((46, 16, 8))
    out["bc/rand_dmr"] = b
    for bnd in (3, 9, 30, 40):
        out[f"bc/dmr_{bnd}"] = unitest.apply_bc_refac(b.copy(), bnd, {"nx": 40, "ny": 10, "x": 4, "y": 1, "dx": 0.1})
    np.savez_compressed(os.path.join(OUT, "drivers.npz"), **out)


def main():
    twin, rie, unitest, dmr = _import_reference()
    make_twin(twin)
    make_drivers(rie, unitest, dmr)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)), "bytes")


if __name__ == "__main__":
    main()
