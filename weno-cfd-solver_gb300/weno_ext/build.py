"""Build libweno_gb300.so (sm_103a) in place, next to this file.

Three translation units are compiled in parallel with nvcc and linked into one
shared library with a C ABI (include/weno_gb300.h):

* csrc/tu_exact.cu -- kernels with --fmad=false (reference-identical doubles)
* csrc/tu_fast.cu  -- kernels with FMA contraction and the FAST forms
* csrc/capi.cu     -- the C entry points and the device-resident solver

Usage: ``python -m weno_ext.build`` (from weno-cfd-solver_gb300/) or
``weno_ext.build.build()``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, "csrc")
LIB_NAME = "libweno_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"] + ARCH

UNITS = {
    "tu_exact.cu": ["--fmad=false"],
    "tu_fast.cu": ["--fmad=true"],
    "tu_df64.cu": ["--fmad=true"],
    "capi.cu": [],
    "probe.cu": [],
    "noalloc.cu": [],
    "batch.cu": ["--fmad=false"],
    "init.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "batch_exact.cu": ["--fmad=false"],
    "batch_f64.cu": ["--fmad=true"],
    "batch_f32.cu": ["--fmad=true"],
}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libweno_gb300.so")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h"))] + [
        os.path.join(PKG_ROOT, "..", "include", "weno_gb300.h")]


def needs_build() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(s) > t for s in _sources() if os.path.exists(s))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB_PATH
    nvcc = _nvcc()
    objdir = os.path.join(PKG_ROOT, "_build")
    os.makedirs(objdir, exist_ok=True)

    def compile_unit(name):
        obj = os.path.join(objdir, name.replace(".cu", ".o"))
        cmd = [nvcc, *COMMON, *UNITS[name], "-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB_PATH + ".tmp"
    r = subprocess.run([nvcc, "-shared", *ARCH, "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
