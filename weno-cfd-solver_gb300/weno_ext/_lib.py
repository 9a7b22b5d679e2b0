"""ctypes binding of libweno_gb300.so (the C ABI declared in include/weno_gb300.h)."""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libweno_gb300.so")

OK, ERR_SHAPE, ERR_ARG, ERR_CUDA, ERR_WORKSPACE, ERR_NUMERIC = range(6)
EXACT, FAST = 0, 1
HLLC, HLLE, BLEND = 0, 1, 2
BC_TRANSMISSIVE, BC_DMR = 0, 1

# Every symbol the header declares, with (restype, argtypes).
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_d = ctypes.c_double
_i = ctypes.c_int
_sz = ctypes.c_size_t
SIGNATURES = {
    "weno_last_error": (ctypes.c_char_p, []),
    "weno_abi_version": (_i, []),
    "weno_flux": (_i, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _d, _i, _i, _vp, _vp]),
    "weno_con2primi": (_i, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _d, _i] + [_vp] * 6 + [_vp]),
    "weno_reconstruct_workspace": (_sz, [_i64, _i64, _i]),
    "weno_reconstruct": (_i, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _d, _i, _i, _i] + [_vp] * 4 + [_vp, _sz, _vp]),
    "weno_riemann_workspace": (_sz, [_i64, _i64, _i]),
    "weno_riemann": (_i, [_vp] * 4 + [_i64, _i64, _d, _i, _i, _d, _d, _i, _vp, _vp, _sz, _vp]),
    "weno_l_local_workspace": (_sz, [_i64, _i64, _i]),
    "weno_l_local": (_i, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _d, _d, _i, _d, _d, _i, _i, _vp, _vp, _sz, _vp]),
    "weno_l_local_host": (_i, [_vp, _i64, _i64, _i64, _d, _d, _i, _d, _d, _i, _i, _vp]),
    "weno_l_local_noalloc": (_i, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _d, _d, _i, _d, _d, _i, _i, _vp, _vp]),
    "weno_solver_create": (_i, [ctypes.POINTER(_vp), _i64, _i64, _d, _d, _i, _i, _i, _i, _d, _d, _d, _d, _i, _i64,
                                _vp, _vp]),
    "weno_solver_destroy": (_i, [_vp]),
    "weno_solver_set_state": (_i, [_vp, _vp, _i64, _i64, _i64, _i64]),
    "weno_solver_set_state_host": (_i, [_vp, _vp, _i64]),
    "weno_solver_run": (_i, [_vp, _i64, _d, _i]),
    "weno_solver_get_state": (_i, [_vp, _vp]),
    "weno_solver_get_state_host": (_i, [_vp, _vp]),
    "weno_solver_info": (_i, [_vp, ctypes.POINTER(_d), ctypes.POINTER(_i64), ctypes.POINTER(_i)]),
    "weno_solver_totals": (_i, [_vp, ctypes.POINTER(_d)]),
    "weno_solver_enable_timing": (_i, [_vp, _i]),
    "weno_solver_timing_report": (_i, [_vp, ctypes.POINTER(_d), ctypes.POINTER(_i64), _i]),
    "weno_solver_launches_per_step": (_i, [_vp]),
    "weno_probe_rates": (_i, [ctypes.POINTER(_d), ctypes.POINTER(_d), ctypes.POINTER(_d), _vp]),
    "weno_fast_math_eval": (_i, [_vp, _vp, _i64, _vp]),
    "weno_init_quadrant": (_i, [_vp, _i64, _i64, _i64, _i64, _vp, _d, _vp]),
    "weno_init_oblique_shock": (_i, [_vp, _i64, _i64, _d, _d, _d, _d, _d, _d, _d, _d, ctypes.POINTER(_i64), _vp,
                                     _vp]),
    "weno_bc_reflecting": (_i, [_vp, _i64, _i64, _i64, _i64, _i64, _i64, _vp]),
    "weno_init_refac": (_i, [_vp, _i64, _i64, _d, _d, _d, ctypes.POINTER(_i64), _vp]),
    "weno_batch_tile_config_count": (_i, []),
    "weno_batch_bytes_per_cell": (_d, [_i, _i, _i]),
    "weno_batch_create": (_i, [ctypes.POINTER(_vp), _i64, _i, _i, _i, _i, _i, _d, _d, _d, _d, _d, _i, _vp]),
    "weno_batch_destroy": (_i, [_vp]),
    "weno_batch_add": (_i, [_vp, _i64, _i64, _d, _i, _i64, _vp, _d, _i64, _d, _vp, _i64, _i64, _i64, _i64,
                            ctypes.POINTER(_i)]),
    "weno_batch_remove": (_i, [_vp, _i]),
    "weno_batch_run": (_i, [_vp, _i64, _i]),
    "weno_batch_get_state": (_i, [_vp, _i, _vp]),
    "weno_batch_info": (_i, [_vp, _i, ctypes.POINTER(_d), ctypes.POINTER(_i64), ctypes.POINTER(_i),
                             ctypes.POINTER(_i)]),
    "weno_batch_poll": (_i, [_vp, _vp, _vp, _vp]),
    "weno_batch_debug_skip_copy": (_i, [_vp, _i, _i64, _i]),
    "weno_batch_stats": (_i, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i)]),
}

_lib = None


class WenoError(RuntimeError):
    """A CUDA-side failure reported by the library."""


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library.  Raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libweno_gb300.so is not built ({LIB_PATH}); run weno_ext.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str):
    if rc == OK:
        return
    msg = load().weno_last_error().decode(errors="replace")
    if rc in (ERR_SHAPE, ERR_ARG, ERR_WORKSPACE):
        raise ValueError(f"{what}: {msg}")
    raise WenoError(f"{what}: {msg}")
