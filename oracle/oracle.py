"""ORACLE -- test infrastructure only (ctypes wrapper of liboracle.so).

CPU restatement of the reference's Rust residual core (weno_ext/src/*.rs) and
of its numpy drivers, used by tests/, the smoke check and bench.py's CPU
baseline leg as the checker.  The product library never imports this module.

The functions mirror the reference's Python-visible names
(weno_ext/src/lib.rs:156-171) so that parity tests read like calls into the
reference: ``flux_x_py``, ``con2primi_py``, ``weno_x_py`` ... ``l_local_py``.
``weno_x_py``/``weno_y_py`` take an extra ``cons`` switch selecting the
component-wise reconstructor that ``l_local`` uses when ``cons_switch`` is set
(weno.rs:635, weno.rs:854).
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_c_dp = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64


def build(force: bool = False) -> str:
    """Compile liboracle.so from weno_oracle.cpp (g++, -ffp-contract=off)."""
    src = os.path.join(_HERE, "weno_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
               "-fopenmp", src, "-o", _LIB_PATH]
        subprocess.run(cmd, check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_set_weno_eps.argtypes = [ctypes.c_double]
        L.orc_set_weno_eps.restype = None
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_threads.restype = ctypes.c_int
        L.orc_flux.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, _i64, ctypes.c_double, ctypes.c_int, _c_dp]
        L.orc_con2primi.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, _i64, ctypes.c_double] + [_c_dp] * 6
        L.orc_reconstruct.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, _i64, ctypes.c_double,
                                      ctypes.c_int, ctypes.c_int] + [_c_dp] * 4
        L.orc_riemann.argtypes = [_c_dp] * 4 + [_i64, _i64, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, _c_dp]
        L.orc_shock_sensor.argtypes = [_c_dp, _i64, _i64, ctypes.c_double, ctypes.c_double, _c_dp]
        L.orc_l_local.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, _i64, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _c_dp]
        L.orc_count_l_local.argtypes = [_c_dp, _i64, _i64, _i64, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_uint64)]
        L.orc_bc_transmissive.argtypes = [_c_dp, _i64, _i64, _i64]
        L.orc_bc_transmissive.restype = None
        L.orc_bc_reflecting.argtypes = [_c_dp, _i64, _i64, _i64]
        L.orc_bc_dmr.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, _i64, _c_dp]
        L.orc_bc_dmr.restype = None
        L.orc_sync_primitives.argtypes = [_c_dp, _i64, _i64, _i64, ctypes.c_double]
        L.orc_sync_primitives.restype = None
        L.orc_cfl_cmax.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, ctypes.c_double]
        L.orc_cfl_cmax.restype = ctypes.c_double
        L.orc_rk3_step.argtypes = [_c_dp, _i64, _i64, _i64, _i64, _i64, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_int, _i64, _c_dp]
        _lib = L
    return _lib


def set_weno_eps(eps: float) -> None:
    """WENO smoothness epsilon of every later call (1e-12 = the reference's DEFAULT_EPS)."""
    lib().orc_set_weno_eps(float(eps))


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def _p(a: np.ndarray):
    return a.ctypes.data_as(_c_dp)


def _view(u: np.ndarray):
    u = np.asarray(u)
    if u.dtype != np.float64 or u.ndim != 3:
        raise TypeError("expected a 3-D float64 array")
    st = [s // 8 for s in u.strides]
    return u, u.shape, st


def _check(rc: int):
    if rc != 0:
        raise ValueError("oracle rejected the input shape")


def flux_x_py(q, gamma):
    u, (m, n, c), (s0, s1, s2) = _view(q)
    out = np.empty((m, n, 4))
    _check(lib().orc_flux(_p(u), m, n, c, s0, s1, s2, gamma, 0, _p(out)))
    return out


def flux_y_py(q, gamma):
    u, (m, n, c), (s0, s1, s2) = _view(q)
    out = np.empty((m, n, 4))
    _check(lib().orc_flux(_p(u), m, n, c, s0, s1, s2, gamma, 1, _p(out)))
    return out


def con2primi_py(q, gamma):
    u, (m, n, c), (s0, s1, s2) = _view(q)
    outs = [np.empty((m, n)) for _ in range(6)]
    _check(lib().orc_con2primi(_p(u), m, n, c, s0, s1, s2, gamma, *[_p(o) for o in outs]))
    return tuple(outs)


def _reconstruct(u, gamma, ydir, cons):
    u, (m, n, c), (s0, s1, s2) = _view(u)
    shape = (m - 6, n - 5, 4) if ydir else (m - 5, n - 6, 4)
    if min(shape) < 0:
        raise ValueError("array too small for a 6-cell stencil")
    outs = [np.empty(shape) for _ in range(4)]
    _check(lib().orc_reconstruct(_p(u), m, n, c, s0, s1, s2, gamma, int(ydir), int(cons), *[_p(o) for o in outs]))
    return tuple(outs)


def weno_x_py(u, gamma, cons=False):
    return _reconstruct(u, gamma, False, cons)


def weno_y_py(u, gamma, cons=False):
    return _reconstruct(u, gamma, True, cons)


def _riemann(q_l, f_l, q_r, f_r, gamma, ydir, kind, jp_lo=0.0, jp_hi=0.0):
    arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64)[:, :, :4]) for a in (q_l, f_l, q_r, f_r)]
    m, n = arrs[0].shape[:2]
    out = np.empty((m, n, 4))
    _check(lib().orc_riemann(*[_p(a) for a in arrs], m, n, gamma, int(ydir), kind, jp_lo, jp_hi, _p(out)))
    return out


def hllc_x_rs_py(q_l, f_l, q_r, f_r, gamma):
    return _riemann(q_l, f_l, q_r, f_r, gamma, False, 0)


def hllc_y_rs_py(q_l, f_l, q_r, f_r, gamma):
    return _riemann(q_l, f_l, q_r, f_r, gamma, True, 0)


def hlle_x_rs_py(q_l, f_l, q_r, f_r, gamma):
    return _riemann(q_l, f_l, q_r, f_r, gamma, False, 1)


def hlle_y_rs_py(q_l, f_l, q_r, f_r, gamma):
    return _riemann(q_l, f_l, q_r, f_r, gamma, True, 1)


def hllc_hlle_x_rs_py(q_l, f_l, q_r, f_r, gamma, jp_lo, jp_hi, force_hlle):
    return _riemann(q_l, f_l, q_r, f_r, gamma, False, 1 if force_hlle else 2, jp_lo, jp_hi)


def hllc_hlle_y_rs_py(q_l, f_l, q_r, f_r, gamma, jp_lo, jp_hi, force_hlle):
    return _riemann(q_l, f_l, q_r, f_r, gamma, True, 1 if force_hlle else 2, jp_lo, jp_hi)


def shock_sensor(p, jp_lo, jp_hi):
    p = np.ascontiguousarray(p, dtype=np.float64)
    out = np.empty_like(p)
    _check(lib().orc_shock_sensor(_p(p), p.shape[0], p.shape[1], jp_lo, jp_hi, _p(out)))
    return out


def l_local_py(u, dx, gamma, force_hlle, jp_cri, cons_switch=False):
    u, (m, n, c), (s0, s1, s2) = _view(u)
    out = np.empty((max(m - 6, 0), max(n - 6, 0), 4))
    jp_lo, jp_hi = (float(x) for x in jp_cri)
    _check(lib().orc_l_local(_p(u), m, n, c, s0, s1, s2, dx, gamma, int(bool(force_hlle)), jp_lo, jp_hi,
                             int(bool(cons_switch)), _p(out)))
    return out


def count_l_local(u, dx, gamma, force_hlle, jp_cri, cons_switch):
    """Exact (add, mul, div, sqrt, cmp) tallies of one l_local call."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    m, n, c = u.shape
    t = (ctypes.c_uint64 * 5)()
    _check(lib().orc_count_l_local(_p(u), m, n, c, dx, gamma, int(force_hlle), float(jp_cri[0]), float(jp_cri[1]),
                                   int(cons_switch), t))
    return dict(zip(("add", "mul", "div", "sqrt", "cmp"), [int(x) for x in t]))


# ---------------------------------------------------------------------------
# Driver arithmetic (in place on a C-contiguous float64 (M, N, C) array).
# ---------------------------------------------------------------------------
DMR_POST = np.array([8, 33, -57.1576, 563.499, 8, 4.125, -7.1447, 116.5], dtype=np.float64)


def _dense(q):
    if not (isinstance(q, np.ndarray) and q.dtype == np.float64 and q.flags.c_contiguous and q.ndim == 3):
        raise TypeError("expected a C-contiguous float64 (M, N, C) array")
    return q


def bc_transmissive(q):
    q = _dense(q)
    lib().orc_bc_transmissive(_p(q), *q.shape)
    return q


def bc_reflecting(q):
    q = _dense(q)
    _check(lib().orc_bc_reflecting(_p(q), *q.shape))
    return q


def bc_dmr(q, nx, ny, bound, post=DMR_POST):
    q = _dense(q)
    post = np.ascontiguousarray(post, dtype=np.float64)
    lib().orc_bc_dmr(_p(q), *q.shape, nx, ny, bound, _p(post))
    return q


def sync_primitives(q, gamma):
    q = _dense(q)
    lib().orc_sync_primitives(_p(q), *q.shape, gamma)
    return q


def cfl_cmax(q, nx, ny, gamma):
    q = _dense(q)
    return lib().orc_cfl_cmax(_p(q), *q.shape, nx, ny, gamma)


def rk3_step(q, nx, ny, dx, dt, gamma, force_hlle, jp_cri, cons, bc="transmissive", bound=0, post=DMR_POST):
    """One SSP-RK3 step, in place (Rie_prob_2d_rs.rk3_cc or double_mach_reflection.rk3_refac)."""
    q = _dense(q)
    post = np.ascontiguousarray(post, dtype=np.float64)
    kind = {"transmissive": 0, "dmr": 1}[bc]
    _check(lib().orc_rk3_step(_p(q), *q.shape, nx, ny, dx, dt, gamma, int(force_hlle), float(jp_cri[0]),
                              float(jp_cri[1]), int(cons), kind, bound, _p(post)))
    return q
