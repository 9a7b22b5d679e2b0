"""Re-enact the reference drivers' recorded calls into weno_ext on a given module.

tests/golden/driver_trace.npz holds, for runs of the unchanged reference drivers
(``Rie_prob_2d_rs.main_rs`` and ``double_mach_reflection.main_rs``), every call
they made into weno_ext: the function, its call form, its scalar arguments and
the SHA-256 digests of the arrays in and out (tests/golden/make_driver_trace.py).

``replay(module, run)`` walks the same time loop -- the drivers' CFL formula,
SSP-RK3 stage arithmetic in numpy's evaluation order, boundary fills and
primitive sync (Rie_prob_2d_rs.py:123-207,285-319; double_mach_reflection.py:
97-134,229-260; unitest.py:207-227) -- feeding each call the arrays produced
from ``module``'s previous results, exactly as the driver would when it imports
``module`` as weno_ext.  Before every call the input digests and the call form
are checked against the trace (so the loop here is the driver's loop, call for
call), and after every call the output digest is checked (so ``module``
returns what the recorded weno_ext returned).  The boundary fills are the
oracle's, which are pinned bit for bit to the reference's own fills.
"""

from __future__ import annotations

import json
import os

import numpy as np

from golden.make_driver_trace import digest

HERE = os.path.dirname(os.path.abspath(__file__))
TRACE = os.path.join(HERE, "golden", "driver_trace.npz")


def load_trace():
    z = np.load(TRACE)
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


class TraceMismatch(AssertionError):
    pass


class _Calls:
    def __init__(self, module, calls):
        self.module = module
        self.calls = calls
        self.k = 0

    def __call__(self, name, *args):
        if self.k >= len(self.calls):
            raise TraceMismatch(f"call {self.k} ({name}) beyond the recorded {len(self.calls)} calls")
        rec = self.calls[self.k]
        where = f"call {self.k} ({rec['fn']})"
        if rec["fn"] != name or rec["npos"] != len(args) or rec["kw"]:
            raise TraceMismatch(f"{where}: the driver called {rec['fn']} with {rec['npos']} positional "
                                f"arguments and keywords {rec['kw']}, the replay {name} with {len(args)}")
        arrays = [a for a in args if isinstance(a, np.ndarray)]
        if [digest(a) for a in arrays] != rec["in"]:
            raise TraceMismatch(f"{where}: input arrays differ from the driver's")
        for k, a in enumerate(args):
            if not isinstance(a, np.ndarray):
                want = rec["scalars"][str(k)]
                got = list(a) if isinstance(a, tuple) else a
                if got != want:
                    raise TraceMismatch(f"{where}: argument {k} is {got!r}, the driver passed {want!r}")
        out = getattr(self.module, name)(*args)
        d = digest(tuple(out) if isinstance(out, (tuple, list)) else out)
        if d != rec["out"]:
            raise TraceMismatch(f"{where}: output differs from the recorded weno_ext's")
        self.k += 1
        return out


def _sync_primitives(call, q, gamma):
    p, a, rho, u, v, h = call("con2primi_py", q, gamma)
    q[:, :, 4] = rho
    q[:, :, 5] = u
    q[:, :, 6] = v
    q[:, :, 7] = p
    return q


def _rk3_cc(call, bc, q, grid, dt, gamma, force_hlle, weno_switch, jp_cri):
    nx, ny, dx = grid["nx"], grid["ny"], grid["dx"]
    sl = np.s_[3:nx + 3, 3:ny + 3, :4]
    bc(q)
    l0 = call("l_local_py", q, dx, gamma, force_hlle, jp_cri, weno_switch)
    q1 = q.copy()
    q1[sl] = q[sl] + dt * l0
    bc(q1)
    _sync_primitives(call, q1, gamma)
    bc(q1)
    l1 = call("l_local_py", q1, dx, gamma, force_hlle, jp_cri, weno_switch)
    q2 = q.copy()
    q2[sl] = 0.75 * q[sl] + 0.25 * q1[sl] + 0.25 * dt * l1
    bc(q2)
    _sync_primitives(call, q2, gamma)
    bc(q2)
    l2 = call("l_local_py", q2, dx, gamma, force_hlle, jp_cri, weno_switch)
    qn = q.copy()
    qn[sl] = (1 / 3) * q[sl] + (2 / 3) * q2[sl] + (2 / 3) * dt * l2
    bc(qn)
    _sync_primitives(call, qn, gamma)
    bc(qn)
    return qn


def _rk3_refac(call, bc, q, grid, dt, gamma, force_hlle, jp_cri):
    nx, ny, dx = grid["nx"], grid["ny"], grid["dx"]
    l0 = call("l_local_py", q, dx, gamma, force_hlle, jp_cri)
    q1 = q.copy()
    q1[3:nx + 3, 3:ny + 3, :4] = q[3:nx + 3, 3:ny + 3, :4] + dt * l0
    q1 = bc(q1)
    l1 = call("l_local_py", q1, dx, gamma, force_hlle, jp_cri)
    q2 = q.copy()
    q2[3:nx + 3, 3:ny + 3, :4] = (0.75 * q[3:nx + 3, 3:ny + 3, :4] + 0.25 * q1[3:nx + 3, 3:ny + 3, :4]
                                  + 0.25 * dt * l1)
    q2 = bc(q2)
    l2 = call("l_local_py", q2, dx, gamma, force_hlle, jp_cri)
    qn = q.copy()
    qn[3:nx + 3, 3:ny + 3, :4] = (1 / 3 * q[3:nx + 3, 3:ny + 3, :4] + 2 / 3 * q2[3:nx + 3, 3:ny + 3, :4]
                                  + 2 / 3 * dt * l2)
    qn = bc(qn)
    p, a, rho_safe, u, v, h = call("con2primi_py", qn, gamma)
    qn[:, :, 4] = rho_safe
    qn[:, :, 5] = u
    qn[:, :, 6] = v
    qn[:, :, 7] = p
    return bc(qn)


def _cmax(q, nx, ny, gamma):
    speed = np.sqrt(q[3:3 + nx, 3:3 + ny, 5] ** 2 + q[3:3 + nx, 3:3 + ny, 6] ** 2)
    c = np.sqrt(gamma * q[3:3 + nx, 3:3 + ny, 7] / np.maximum(q[3:3 + nx, 3:3 + ny, 0], 1e-14))
    return float(np.max(c + speed))


def replay(module, run, gamma=1.4):
    """Run the recorded driver loop of `run` with `module` as weno_ext; returns the final
    array and the number of calls checked.  Raises TraceMismatch at the first difference."""
    from oracle import oracle
    z, meta = load_trace()
    m = meta[run]
    call = _Calls(module, m["calls"])
    grid, ctrl = m["grid"], m["control"]
    q = np.array(z[f"{run}/first_input"])
    jp = tuple(ctrl["jp_cri"])
    cfl = float(ctrl["CFL"])
    nx, ny, dx = int(grid["nx"]), int(grid["ny"]), float(grid["dx"])
    if m["driver"] == "rie":
        bc = oracle.bc_transmissive
        for _ in range(int(ctrl["nstep"])):
            dt = cfl * dx / (_cmax(q, nx, ny, gamma) + 1e-16)
            q = _rk3_cc(call, bc, q, grid, dt, gamma, bool(ctrl["force_hlle"]), bool(ctrl["weno type"]), jp)
    else:
        bound = _dmr_bound(grid)
        bc = lambda a: oracle.bc_dmr(a, nx, ny, bound)  # noqa: E731
        t_final, T, step, max_steps = float(ctrl["t_final"]), 0.0, 0, int(ctrl["nstep"])
        while T < t_final - 1e-12 and step < max_steps:
            dt = min(cfl * dx / (_cmax(q, nx, ny, gamma) + 1e-16), t_final - T)
            q = _rk3_refac(call, bc, q, grid, dt, gamma, ctrl["force_hlle"], jp)
            T += dt
            step += 1
    if call.k != len(m["calls"]):
        raise TraceMismatch(f"the replay made {call.k} calls, the driver {len(m['calls'])}")
    if digest(q) != m["final"]:
        raise TraceMismatch("final array differs from the one the driver returned")
    return q, call.k


def _dmr_bound(grid):
    """unitest.init_refac's `bound`: the last padded row whose shock-line height rounds to
    the wall (unitest.py:184-193)."""
    nx, ny, lx, ly = grid["nx"], grid["ny"], grid["x"], grid["y"]
    bound = 0
    for i in range(3, nx + 3):
        x = (i - 3 + 0.5) / nx * lx
        y = np.sqrt(3) * x - np.sqrt(3) / 6
        if int(np.round(y / ly * ny)) == 0:
            bound = i
    return bound
