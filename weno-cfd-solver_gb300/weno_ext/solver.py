"""Device-resident SSP-RK3 solver (the time loop of the reference drivers, on the GPU).

One object holds one 2-D problem: the conserved state as four planes of
(nx+6) x (ny+6) in HBM, two stage buffers, the residual workspace and a small
control block (dt, time, step count).  A step is the sequence of the driver's
``rk3_cc`` (Rie_prob_2d_rs.py:169-207) or ``rk3_refac``
(double_mach_reflection.py:97-134): CFL reduction and dt (Rie_prob_2d_rs.py:
311-319), boundary fill, three residual evaluations each fused with its stage
combination, boundary fills -- all on the device, captured once as a CUDA graph
and replayed.  In t_final mode the loop condition is evaluated on the device,
so a batch of steps can be enqueued without host round trips.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

# unitest.py:215 -- the inflow state of the oblique-shock boundary.
DMR_POST = (8.0, 33.0, -57.1576, 563.499, 8.0, 4.125, -7.1447, 116.5)


class Solver:
    def __init__(self, nx, ny, dx, gamma=1.4, *, precision=64, mode="exact", cons=False, force_hlle=True,
                 jp_cri=(0.2, 1.0), cfl=0.5, bc="transmissive", bound=0, post=None, device=None, weno_eps=1e-12):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("Solver needs a CUDA GPU; there is no CPU fallback")
        self._torch = torch
        self.L = _lib.load()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.nx, self.ny, self.dx, self.gamma = int(nx), int(ny), float(dx), float(gamma)
        self.M, self.N = self.nx + 6, self.ny + 6
        self.precision = {"df64": 48, "f64": 64, "f32": 32}.get(precision, precision)
        self.precision = int(self.precision)
        self.bc = bc
        bc_kind = {"transmissive": _lib.BC_TRANSMISSIVE, "dmr": _lib.BC_DMR}[bc]
        post8 = np.ascontiguousarray(DMR_POST if post is None else post, dtype=np.float64)
        if post8.shape != (8,):
            raise ValueError("post must hold the 8 channels of the inflow state")
        with torch.cuda.device(self.device):
            self.stream = torch.cuda.Stream()
        h = ctypes.c_void_p()
        _lib.check(self.L.weno_solver_create(
            ctypes.byref(h), self.nx, self.ny, self.dx, self.gamma, self.precision,
            _lib.FAST if mode == "fast" else _lib.EXACT, int(bool(cons)), int(bool(force_hlle)),
            float(jp_cri[0]), float(jp_cri[1]), float(cfl), float(weno_eps), bc_kind, int(bound), post8.ctypes.data,
            self.stream.cuda_stream), "Solver")
        self._h = h

    # -- state -------------------------------------------------------------
    def set_state(self, q):
        """Load (nx+6, ny+6, C>=4) float64 from a numpy array (host) or a torch CUDA tensor.
        With C >= 8 the first dt uses the primitive channels 5..7, as the driver's CFL does."""
        torch = self._torch
        if isinstance(q, torch.Tensor):
            if q.shape[:2] != (self.M, self.N) or q.dtype != torch.float64 or not q.is_cuda:
                raise ValueError(f"state must be a float64 CUDA tensor of shape ({self.M}, {self.N}, C)")
            self.stream.wait_stream(torch.cuda.current_stream())
            s = q.stride()
            _lib.check(self.L.weno_solver_set_state(self._h, q.data_ptr(), q.shape[2], s[0], s[1], s[2]),
                       "set_state")
        else:
            a = np.ascontiguousarray(q, dtype=np.float64)
            if a.ndim != 3 or a.shape[:2] != (self.M, self.N):
                raise ValueError(f"state must have shape ({self.M}, {self.N}, C)")
            _lib.check(self.L.weno_solver_set_state_host(self._h, a.ctypes.data, a.shape[2]), "set_state")

    def state(self, device=False):
        """The driver's (nx+6, ny+6, 8) array: conserved channels, then rho_safe, u, v, p."""
        torch = self._torch
        if device:
            out = torch.empty((self.M, self.N, 8), dtype=torch.float64, device=self.device)
            _lib.check(self.L.weno_solver_get_state(self._h, out.data_ptr()), "state")
            torch.cuda.current_stream().wait_stream(self.stream)
            return out
        out = np.empty((self.M, self.N, 8))
        _lib.check(self.L.weno_solver_get_state_host(self._h, out.ctypes.data), "state")
        return out

    # -- time loop ---------------------------------------------------------
    def run(self, nsteps, t_final=None, graph=True):
        """Enqueue ``nsteps`` steps (asynchronous).  With t_final, steps past the end time are
        device-side no-ops and dt is clipped to the time left."""
        _lib.check(self.L.weno_solver_run(self._h, int(nsteps), -1.0 if t_final is None else float(t_final),
                                          int(bool(graph))), "run")

    def info(self):
        t = ctypes.c_double()
        n = ctypes.c_int64()
        st = ctypes.c_int()
        _lib.check(self.L.weno_solver_info(self._h, ctypes.byref(t), ctypes.byref(n), ctypes.byref(st)), "info")
        return t.value, n.value, st.value

    def totals(self):
        """FP64 sums of rho, rho*u, rho*v, E over the interior cells."""
        out = (ctypes.c_double * 4)()
        _lib.check(self.L.weno_solver_totals(self._h, out), "totals")
        return tuple(out)

    @property
    def t(self):
        return self.info()[0]

    @property
    def steps(self):
        return self.info()[1]

    def synchronize(self):
        self.stream.synchronize()

    @property
    def launches_per_step(self):
        return self.L.weno_solver_launches_per_step(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self.L.weno_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
