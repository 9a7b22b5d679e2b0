"""CPU checks of the drop-in boundary: the library builds, loads and exports every
symbol include/weno_gb300.h declares; the Python module exposes the reference's
twelve functions with the reference's argument order; without a GPU a call fails
loudly instead of falling back to the CPU."""

import ctypes
import inspect
import os
import re

import pytest

from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "weno_gb300.h")

# lib.rs:156-171 registration order, with lib.rs's positional parameters.
REFERENCE_API = {
    "flux_x_py": ["q", "gamma"],
    "flux_y_py": ["q", "gamma"],
    "con2primi_py": ["q", "gamma"],
    "weno_x_py": ["u", "gamma"],
    "weno_y_py": ["u", "gamma"],
    "hllc_x_rs_py": ["q_l", "f_l", "q_r", "f_r", "gamma"],
    "hllc_y_rs_py": ["q_l", "f_l", "q_r", "f_r", "gamma"],
    "hlle_x_rs_py": ["q_l", "f_l", "q_r", "f_r", "gamma"],
    "hlle_y_rs_py": ["q_l", "f_l", "q_r", "f_r", "gamma"],
    "hllc_hlle_x_rs_py": ["q_l", "f_l", "q_r", "f_r", "gamma", "jp_lo", "jp_hi", "force_hlle"],
    "hllc_hlle_y_rs_py": ["q_l", "f_l", "q_r", "f_r", "gamma", "jp_lo", "jp_hi", "force_hlle"],
    "l_local_py": ["u", "dx", "gamma", "force_hlle", "jp_cri", "cons_switch"],
}


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(weno_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = header_functions()
    for must in ("weno_l_local", "weno_reconstruct", "weno_riemann", "weno_flux", "weno_con2primi",
                 "weno_solver_create", "weno_solver_run"):
        assert must in names


def test_library_builds_and_exports_every_declared_symbol():
    from weno_ext import _lib, build
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in header_functions():
        assert hasattr(lib, name), f"{name} declared in weno_gb300.h but not exported"
    # and the ctypes binding covers exactly the declared functions
    assert sorted(_lib.SIGNATURES) == header_functions()
    L = _lib.load()
    assert L.weno_abi_version() == 2


def test_reference_api_surface():
    import weno_ext
    for name, params in REFERENCE_API.items():
        fn = getattr(weno_ext, name)
        got = list(inspect.signature(fn).parameters)
        assert got[: len(params)] == params, f"{name}: {got} != {params}"
    sig = inspect.signature(weno_ext.l_local_py)
    assert sig.parameters["cons_switch"].default is False  # five-argument callers (double_mach_reflection.py:62)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback_without_gpu():
    import numpy as np
    import weno_ext
    q = np.ones((10, 10, 8))
    with pytest.raises(RuntimeError):
        weno_ext.l_local_py(q, 0.1, 1.4, True, (0.2, 1.0), True)
    with pytest.raises(RuntimeError):
        weno_ext.flux_x_py(q, 1.4)
