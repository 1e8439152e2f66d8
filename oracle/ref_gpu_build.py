"""Builds the reference's own CUDA kernels for sm_103a -- TEST INFRASTRUCTURE.

The reference keeps every step kernel in one header of templates
(maxwell_solver src/gpu.h, instantiated with float through `typedef float
real`, src/simulation.h:15).  This script compiles that header, unchanged and
where it lies, with NVRTC into a cubin for sm_103a, and records the lowered
(mangled) name of each float instantiation, so that tests/refgpu.py can load
the cubin through the CUDA driver API and launch the reference's kernels with
the reference's launch shapes.  Nothing here is copied from the reference:
the source handed to NVRTC is one #include line.

Two builds:
  ref_gpu.cubin        the reference's flags: nvcc's defaults (fused
                       multiply-add contraction on), src/Compile.m:4-6;
  ref_gpu_nofma.cubin  the same with contraction off, which is how the
                       library's kernels and the CPU oracle evaluate every
                       expression.
Outputs go to oracle/_ref/ (kept out of history, carried to the GPU machine with
the rest of the tree); the reference's sources are read, never written.

    python oracle/ref_gpu_build.py [REFERENCE_ROOT]

REFERENCE_ROOT (or $MAXWELL_REF) is the reference checkout holding src/gpu.h.
"""
from __future__ import annotations

import ctypes
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# The float instantiations the step loop launches: the 3D curl updates, the
# CPML corrections and the TF/SF face kernels of the four reachable modes
# (src/simulation.h:330-570), plus the current source (:256-286).
KERNELS = [
    "GPU_updateH", "GPU_updateE",
    "GPU_updateHPmlX", "GPU_updateHPmlY", "GPU_updateHPmlZ",
    "GPU_updateEPmlX", "GPU_updateEPmlY", "GPU_updateEPmlZ",
    "GPU_updateHx_PlaneWaveZ_Y", "GPU_updateHz_PlaneWaveZ_Y",
    "GPU_updateEy_PlaneWaveZ_Y", "GPU_updateEz_PlaneWaveZ_Y",
    "GPU_updateHy_PlaneWaveZ_X", "GPU_updateHz_PlaneWaveZ_X",
    "GPU_updateEx_PlaneWaveZ_X", "GPU_updateEz_PlaneWaveZ_X",
    "GPU_updateHx_PlaneWaveX_Z", "GPU_updateHy_PlaneWaveX_Z",
    "GPU_updateEx_PlaneWaveX_Z", "GPU_updateEz_PlaneWaveX_Z",
    "GPU_updateHx_PlaneWaveX_Y", "GPU_updateHz_PlaneWaveX_Y",
    "GPU_updateEx_PlaneWaveX_Y", "GPU_updateEy_PlaneWaveX_Y",
    "AddSource_GPU_3D_1DThread",
]
ARCH = "sm_103a"


def _nvrtc():
    cands = []
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for d in ("lib64", "lib", "targets/x86_64-linux/lib", "targets/sbsa-linux/lib"):
        cands += sorted(glob.glob(os.path.join(home, d, "libnvrtc.so*")))
    for c in cands + ["libnvrtc.so"]:
        try:
            return ctypes.CDLL(c)
        except OSError:
            continue
    raise RuntimeError("libnvrtc not found")


def _check(lib, rc, what, prog=None):
    if rc == 0:
        return
    log = ""
    if prog is not None:
        n = ctypes.c_size_t(0)
        lib.nvrtcGetProgramLogSize(prog, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value + 1)
        lib.nvrtcGetProgramLog(prog, buf)
        log = buf.value.decode(errors="replace")
    lib.nvrtcGetErrorString.restype = ctypes.c_char_p
    raise RuntimeError(f"{what}: {lib.nvrtcGetErrorString(rc).decode()}\n{log}")


def build_one(src_dir: str, fmad: bool, cuda_include: str):
    """(cubin bytes, {kernel: lowered name}) of one NVRTC build."""
    lib = _nvrtc()
    prog = ctypes.c_void_p()
    source = b'#include "gpu.h"\n'
    # the runtime headers gpu.h names are host-side; NVRTC provides the
    # device built-ins itself, so they are given as empty headers
    hdr_names = (ctypes.c_char_p * 2)(b"cuda_runtime.h", b"device_launch_parameters.h")
    hdr_src = (ctypes.c_char_p * 2)(b"", b"")
    _check(lib, lib.nvrtcCreateProgram(ctypes.byref(prog), source, b"ref_gpu.cu", 2, hdr_src,
                                       hdr_names), "nvrtcCreateProgram")
    exprs = [f"{k}<float>".encode() for k in KERNELS]
    for e in exprs:
        _check(lib, lib.nvrtcAddNameExpression(prog, e), "nvrtcAddNameExpression")
    opts = [f"--gpu-architecture={ARCH}".encode(), b"--std=c++17",
            f"--fmad={'true' if fmad else 'false'}".encode(),
            f"-I{src_dir}".encode(), f"-I{cuda_include}".encode()]
    arr = (ctypes.c_char_p * len(opts))(*opts)
    _check(lib, lib.nvrtcCompileProgram(prog, len(opts), arr), "nvrtcCompileProgram", prog)
    n = ctypes.c_size_t(0)
    _check(lib, lib.nvrtcGetCUBINSize(prog, ctypes.byref(n)), "nvrtcGetCUBINSize")
    buf = ctypes.create_string_buffer(n.value)
    _check(lib, lib.nvrtcGetCUBIN(prog, buf), "nvrtcGetCUBIN")
    names = {}
    for k, e in zip(KERNELS, exprs):
        low = ctypes.c_char_p()
        _check(lib, lib.nvrtcGetLoweredName(prog, e, ctypes.byref(low)), "nvrtcGetLoweredName")
        names[k] = low.value.decode()
    lib.nvrtcDestroyProgram(ctypes.byref(prog))
    return buf.raw, names


def build(ref_root: str | None = None) -> None:
    ref_root = ref_root or os.environ.get("MAXWELL_REF")
    if not ref_root:
        raise SystemExit("usage: ref_gpu_build.py REFERENCE_ROOT (or set MAXWELL_REF)")
    src_dir = os.path.join(ref_root, "src")
    if not os.path.isfile(os.path.join(src_dir, "gpu.h")):
        raise SystemExit(f"{src_dir}/gpu.h not found")
    cuda_include = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    os.makedirs(OUT, exist_ok=True)
    meta = {"arch": ARCH, "kernels": {}}
    for fmad, fname in ((True, "ref_gpu.cubin"), (False, "ref_gpu_nofma.cubin")):
        cubin, names = build_one(src_dir, fmad, cuda_include)
        with open(os.path.join(OUT, fname), "wb") as f:
            f.write(cubin)
        meta["kernels"] = names  # the same names in both builds
    with open(os.path.join(OUT, "ref_gpu_names.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else None)
