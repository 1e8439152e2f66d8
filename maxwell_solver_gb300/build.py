"""In-tree build of libfdtd_gb300.so for sm_103a (GB300).

nvcc compiles the kernels (one -gencode, --fmad=false so every float
operation is rounded separately, as in the reference order), gcc compiles
the C host, nvcc links (static cudart).  Output:
maxwell_solver_gb300/lib/libfdtd_gb300.so.  Rebuilds only when a source is
newer than the library.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(LIB_DIR, "libfdtd_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    c = sorted(glob.glob(os.path.join(CSRC, "*.c")))
    hdr = (sorted(glob.glob(os.path.join(CSRC, "*.h"))) + sorted(glob.glob(os.path.join(CSRC, "*.cuh")))
           + [os.path.join(INCLUDE, "fdtd_gb300.h")])
    return cu, c, hdr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _defines() -> str:
    return " ".join(os.environ.get("FDTD_NVCC_DEFINES", "").split())


def _stamp_ok() -> bool:
    """The library was built with the current FDTD_NVCC_DEFINES."""
    try:
        with open(LIB + ".defines") as f:
            return f.read() == _defines()
    except OSError:
        return _defines() == ""


def build(force: bool = False, verbose: bool = False) -> str:
    cu, c, hdr = _sources()
    if not force and _stamp_ok() and not _stale(LIB, cu + c + hdr + [__file__]):
        return LIB
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(OBJ_DIR, exist_ok=True)
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{os.path.join(home, 'include')}"]
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append([nvcc, ARCH, "-lineinfo", "-O3", "--fmad=false", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                     *inc, *_defines().split(), "-c", src, "-o", obj])
    for src in c:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off",
                     "-Wall", "-Wno-unused-function", *inc, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    tmp = LIB + f".tmp{os.getpid()}"
    run([nvcc, ARCH, "-shared", "-o", tmp, *objs, "-lpthread", "-lm"])
    os.replace(tmp, LIB)
    with open(LIB + ".defines", "w") as f:
        f.write(_defines())
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
