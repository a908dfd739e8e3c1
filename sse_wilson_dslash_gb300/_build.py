"""Build the native libraries in-tree (no cmake, no torch extension machinery).

    libgbdslash.so    CUDA kernels (sm_103a) + extended C ABI (include/gbdslash.h)
    libgbdslash32.so  drop-in: the reference's entry points, SSEREAL = float
    libgbdslash64.so  drop-in: the reference's entry points, SSEREAL = double

The .cu translation units compile in parallel; outputs go to
``sse_wilson_dslash_gb300/lib`` (libraries) and ``sse_wilson_dslash_gb300/_build``
(objects).  A step is skipped when its outputs are newer than its inputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC] + ARCH


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose: bool = False, jobs: int | None = None) -> dict:
    """Compile everything that is out of date; return paths of the libraries."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs, todo = [], []
    for s in sources:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            todo.append([nvcc(), *NVCC_FLAGS, "-c", s, "-o", o])
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, todo):
                if verbose and r.stderr:
                    print(r.stderr)
    core = os.path.join(LIB, "libgbdslash.so")
    if _stale(core, objs):
        _run([nvcc(), "-shared", *ARCH, "-o", core, *objs, "-Xlinker", "-soname=libgbdslash.so"])
    shim = os.path.join(CSRC, "legacy_shim.c")
    out = {"core": core}
    for prec in (32, 64):
        lib = os.path.join(LIB, f"libgbdslash{prec}.so")
        if _stale(lib, [shim, core] + headers):
            _run(["gcc", "-O2", "-fPIC", "-shared", f"-DGBDS_SHIM_PREC={prec}", "-I" + INCLUDE, shim,
                  "-L" + LIB, "-lgbdslash", "-Wl,-rpath,$ORIGIN", "-o", lib])
        out[f"legacy{prec}"] = lib
    return out


if __name__ == "__main__":
    print(build(verbose=True))
