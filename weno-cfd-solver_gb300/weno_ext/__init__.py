"""weno_ext -- GB300 (sm_103a) drop-in for the reference's Rust extension.

Exports the twelve functions of the reference module (weno_ext/src/lib.rs:156-171,
declared in weno_ext/weno_ext.pyi) with the same positional order and
meaning, so that Rie_prob_2d_rs.py, double_mach_reflection.py and the other
drivers import this package unchanged.  Every call runs hand-written CUDA
kernels through the C ABI of libweno_gb300.so; there is no CPU fallback, and
importing works without a GPU but calling raises RuntimeError.

Arrays:
* numpy float64 3-D arrays in -> new numpy arrays out (host copies in and out;
  the call returns when the result is on the host), as the reference does;
* torch float64 CUDA tensors in -> torch CUDA tensors out on the same device,
  enqueued on the current torch stream (asynchronous, like any torch op).

Inputs are never modified.  Only channels 0..3 (rho, rho*u, rho*v, E) are read;
arrays need at least 4 channels (the reference asserts c >= 4, weno.rs:371).

Arithmetic: ``set_mode("exact")`` (default) reproduces the Rust core's IEEE
doubles bit for bit; ``set_mode("fast")`` (or WENO_EXT_MODE=fast) uses the
reformulated kernels with fewer FP64 operations, equal to rounding (about
1e-16 relative L1 on a step, within 1e-10 over multi-step runs).
"""

from __future__ import annotations

import os
import warnings

import numpy as np

from . import _lib
from ._lib import WenoError

__all__ = [
    "flux_x_py", "flux_y_py", "con2primi_py", "weno_x_py", "weno_y_py", "hllc_x_rs_py", "hllc_y_rs_py",
    "hlle_x_rs_py", "hlle_y_rs_py", "hllc_hlle_x_rs_py", "hllc_hlle_y_rs_py", "l_local_py",
    "set_mode", "get_mode", "Solver", "Batch", "WenoError", "library_path",
]

_MODE = _lib.FAST if os.environ.get("WENO_EXT_MODE", "exact").lower() == "fast" else _lib.EXACT


def set_mode(mode: str) -> None:
    """Select the arithmetic policy: "exact" (bit-identical to the Rust core) or "fast"."""
    global _MODE
    m = mode.lower()
    if m not in ("exact", "fast"):
        raise ValueError("mode must be 'exact' or 'fast'")
    _MODE = _lib.EXACT if m == "exact" else _lib.FAST


def get_mode() -> str:
    return "exact" if _MODE == _lib.EXACT else "fast"


def library_path() -> str:
    return _lib.LIB_PATH


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("weno_ext runs on a CUDA GPU (sm_103a); no GPU is visible and there is no CPU fallback")
    _lib.load()
    return torch


class _In:
    """One array argument, resident on the device for the call."""

    __slots__ = ("t", "host", "shape", "strides")

    def __init__(self, x, name, torch, channels4=False):
        if isinstance(x, torch.Tensor):
            if not x.is_cuda:
                raise TypeError(f"{name}: torch tensors must be on a CUDA device")
            if x.dtype != torch.float64:
                raise TypeError(f"{name}: expected float64, got {x.dtype}")
            if x.dim() != 3:
                raise TypeError(f"{name}: expected a 3-D array, got {x.dim()}-D")
            t = x[:, :, :4].contiguous() if channels4 else x
            self.host = False
        else:
            if not isinstance(x, np.ndarray):
                raise TypeError(f"{name}: expected a numpy.ndarray or a torch CUDA tensor, got {type(x).__name__}")
            if x.dtype != np.float64:
                raise TypeError(f"{name}: expected float64, got {x.dtype}")
            if x.ndim != 3:
                raise TypeError(f"{name}: expected a 3-D array, got {x.ndim}-D")
            a = np.ascontiguousarray(x[:, :, :4] if channels4 else x)
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                t = torch.from_numpy(a).to(torch.cuda.current_device())
            self.host = True
        if t.shape[2] < 4:
            raise ValueError(f"{name}: needs at least 4 channels, got {t.shape[2]}")
        self.t = t
        self.shape = tuple(t.shape)
        self.strides = tuple(t.stride())

    @property
    def ptr(self):
        return self.t.data_ptr()


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


def _empty(torch, shape):
    return torch.empty(shape, dtype=torch.float64, device=torch.cuda.current_device())


def _out(res, host):
    if host:
        return tuple(r.cpu().numpy() for r in res) if isinstance(res, tuple) else res.cpu().numpy()
    return res


def _flux(q, gamma, ydir):
    torch = _torch()
    a = _In(q, "q", torch)
    m, n, c = a.shape
    out = _empty(torch, (m, n, 4))
    _lib.check(_lib.load().weno_flux(a.ptr, m, n, c, *a.strides, float(gamma), ydir, _MODE, out.data_ptr(),
                                     _stream(torch)), "flux")
    return _out(out, a.host)


def flux_x_py(q, gamma):
    """Euler flux normal to x of channels 0..3 (lib.rs:18-23, utils.rs:74-90)."""
    return _flux(q, gamma, 0)


def flux_y_py(q, gamma):
    """Euler flux normal to y (lib.rs:25-30, utils.rs:93-109)."""
    return _flux(q, gamma, 1)


def con2primi_py(q, gamma):
    """(p, a, rho, u, v, h) with clamped density and pressure (lib.rs:32-38, utils.rs:9-35)."""
    torch = _torch()
    a = _In(q, "q", torch)
    m, n, c = a.shape
    outs = tuple(_empty(torch, (m, n)) for _ in range(6))
    _lib.check(_lib.load().weno_con2primi(a.ptr, m, n, c, *a.strides, float(gamma), _MODE,
                                          *[o.data_ptr() for o in outs], _stream(torch)), "con2primi")
    return _out(outs, a.host)


def _reconstruct(u, gamma, ydir, cons):
    torch = _torch()
    a = _In(u, "u", torch)
    m, n, c = a.shape
    if m < 6 or n < 6:
        raise ValueError(f"u: needs at least 6 x 6 cells for the WENO stencils, got {m} x {n}")
    shape = (m - 6, n - 5, 4) if ydir else (m - 5, n - 6, 4)
    outs = tuple(_empty(torch, shape) for _ in range(4))
    L = _lib.load()
    wsb = L.weno_reconstruct_workspace(m, n, ydir)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=torch.cuda.current_device())
    _lib.check(L.weno_reconstruct(a.ptr, m, n, c, *a.strides, float(gamma), ydir, int(bool(cons)), _MODE,
                                  *[o.data_ptr() for o in outs], ws.data_ptr(), wsb, _stream(torch)), "weno")
    return _out(outs, a.host)


def weno_x_py(u, gamma, cons=False):
    """WENO5 + Gauss-quadrature face states and fluxes normal to x: (q_l, f_l, q_r, f_r), each
    (m-5, n-6, 4).  Characteristic projection as the reference's weno_x_py (lib.rs:40-45,
    weno.rs:367-502); ``cons=True`` gives the component-wise variant l_local uses (weno.rs:635-852)."""
    return _reconstruct(u, gamma, 0, cons)


def weno_y_py(u, gamma, cons=False):
    """As weno_x_py for faces normal to y, each (m-6, n-5, 4) (lib.rs:47-52, weno.rs:508-632)."""
    return _reconstruct(u, gamma, 1, cons)


def _riemann(q_l, f_l, q_r, f_r, gamma, ydir, kind, jp_lo=0.0, jp_hi=0.0):
    torch = _torch()
    args = [_In(x, nm, torch, channels4=True) for x, nm in ((q_l, "q_l"), (f_l, "f_l"), (q_r, "q_r"), (f_r, "f_r"))]
    m, n = args[0].shape[:2]
    for a, nm in zip(args, ("q_l", "f_l", "q_r", "f_r")):
        if a.shape[:2] != (m, n):
            raise ValueError(f"{nm}: shape {a.shape[:2]} differs from q_l's {(m, n)}")
    out = _empty(torch, (m, n, 4))
    L = _lib.load()
    wsb = L.weno_riemann_workspace(m, n, kind)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=torch.cuda.current_device())
    _lib.check(L.weno_riemann(*[a.ptr for a in args], m, n, float(gamma), ydir, kind, float(jp_lo), float(jp_hi),
                              _MODE, out.data_ptr(), ws.data_ptr(), wsb, _stream(torch)), "riemann")
    return _out(out, args[0].host)


def hllc_x_rs_py(q_l, f_l, q_r, f_r, gamma):
    """HLLC interface flux normal to x (lib.rs:54-63, riemann.rs:6-96)."""
    return _riemann(q_l, f_l, q_r, f_r, gamma, 0, _lib.HLLC)


def hllc_y_rs_py(q_l, f_l, q_r, f_r, gamma):
    """HLLC interface flux normal to y (lib.rs:65-74, riemann.rs:99-189)."""
    return _riemann(q_l, f_l, q_r, f_r, gamma, 1, _lib.HLLC)


def hlle_x_rs_py(q_l, f_l, q_r, f_r, gamma):
    """HLLE interface flux normal to x (lib.rs:76-85, riemann.rs:191-269)."""
    return _riemann(q_l, f_l, q_r, f_r, gamma, 0, _lib.HLLE)


def hlle_y_rs_py(q_l, f_l, q_r, f_r, gamma):
    """HLLE interface flux normal to y (lib.rs:87-96, riemann.rs:271-349)."""
    return _riemann(q_l, f_l, q_r, f_r, gamma, 1, _lib.HLLE)


def hllc_hlle_x_rs_py(q_l, f_l, q_r, f_r, gamma, jp_lo, jp_hi, force_hlle):
    """HLLE if force_hlle, else the pressure-gradient HLLC/HLLE blend (lib.rs:98-115,
    riemann.rs:352-448)."""
    return _riemann(q_l, f_l, q_r, f_r, gamma, 0, _lib.HLLE if force_hlle else _lib.BLEND, jp_lo, jp_hi)


def hllc_hlle_y_rs_py(q_l, f_l, q_r, f_r, gamma, jp_lo, jp_hi, force_hlle):
    """As hllc_hlle_x_rs_py for faces normal to y (lib.rs:117-132, riemann.rs:450-486)."""
    return _riemann(q_l, f_l, q_r, f_r, gamma, 1, _lib.HLLE if force_hlle else _lib.BLEND, jp_lo, jp_hi)


def l_local_py(u, dx, gamma, force_hlle, jp_cri, cons_switch=False):
    """Residual -(dF/dx + dG/dy) of u (nx+6, ny+6, C>=4) -> (nx, ny, 4) (lib.rs:134-153,
    riemann.rs:489-541).  ``cons_switch`` selects the component-wise reconstruction; it defaults
    to False (characteristic) so that five-argument callers such as
    double_mach_reflection.py:62 run."""
    torch = _torch()
    jp = tuple(jp_cri)
    if len(jp) != 2:
        raise TypeError("jp_cri must hold two numbers (jp_lo, jp_hi)")
    L = _lib.load()
    fh = int(bool(force_hlle))
    if not isinstance(u, torch.Tensor):
        if not isinstance(u, np.ndarray) or u.dtype != np.float64 or u.ndim != 3:
            raise TypeError("u: expected a 3-D float64 numpy.ndarray or torch CUDA tensor")
        a = np.ascontiguousarray(u)
        m, n, c = a.shape
        out = np.empty((max(m - 6, 0), max(n - 6, 0), 4))
        _lib.check(L.weno_l_local_host(a.ctypes.data, m, n, c, float(dx), float(gamma), fh, float(jp[0]),
                                       float(jp[1]), int(bool(cons_switch)), _MODE, out.ctypes.data), "l_local")
        return out
    a = _In(u, "u", torch)
    m, n, c = a.shape
    out = _empty(torch, (max(m - 6, 0), max(n - 6, 0), 4))
    wsb = L.weno_l_local_workspace(m, n, fh)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=u.device)
    _lib.check(L.weno_l_local(a.ptr, m, n, c, *a.strides, float(dx), float(gamma), fh, float(jp[0]), float(jp[1]),
                              int(bool(cons_switch)), _MODE, out.data_ptr(), ws.data_ptr(), wsb, _stream(torch)),
               "l_local")
    return out


from .solver import Solver  # noqa: E402
from .batch import Batch  # noqa: E402
