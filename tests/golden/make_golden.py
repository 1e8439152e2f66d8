"""Generates tests/golden/*.npz from the reference itself.

Runs every scenario of tests/scenarios.py through the reference's own
mexFunction (src/simFDTD.cu + src/simulation.h + src/gpu.h, built for the
host by oracle/ref_build.sh into oracle/_ref/libref_fdtd.so, driven through
tests/mexstub) and stores, per scenario:

  in_*      the exact inputs (freqRes, TimeDim, sources, materials)
  sha_*     sha256 of each float32 output array (fields, psi, coefficients,
            1D incident tables) -- the bit-exact pin
  norm_*    L2 norm (float64) of each array
  smp_*     512 seeded samples (index, value) of each 3D array
  b_E/c_E/b_H/c_H, den_ex (x row), Chh/Che   the CPML / coefficient tables

Needs the reference sources (this container); the GPU machine uses the
committed .npz files only.  Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from mexstub.mexdrv import MexDriver  # noqa: E402
from scenarios import SCENARIOS, run_mex  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
FIELD_NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
PSI_NAMES = ("psi_Exy", "psi_Ezy", "psi_Hxy", "psi_Hzy", "psi_Exz", "psi_Eyz",
             "psi_Hxz", "psi_Hyz", "psi_Eyx", "psi_Ezx", "psi_Hyx", "psi_Hzx")
COEF_NAMES = ("Cexe", "Ceye", "Ceze", "Cexh", "Ceyh", "Cezh")
TABLE_NAMES = ("Ez_1D", "Hy_1D", "E_inv_1D", "H_inv_1D")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def main():
    lib = oracle.build_reference()
    if lib is None:
        raise SystemExit("reference sources not found; cannot regenerate golden vectors")
    drv = MexDriver(lib, "ref_mexFunction")
    drv.lib.ref_array.restype = ctypes.POINTER(ctypes.c_float)
    drv.lib.ref_array.argtypes = [ctypes.c_uint64, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
    drv.lib.ref_scalar.restype = ctypes.c_double
    drv.lib.ref_scalar.argtypes = [ctypes.c_uint64, ctypes.c_char_p]

    def ref_array(P, name):
        cnt = ctypes.c_size_t(0)
        ptr = drv.lib.ref_array(int(P[0]), name.encode(), ctypes.byref(cnt))
        if not ptr or cnt.value == 0:
            return None
        return np.ctypeslib.as_array(ptr, shape=(cnt.value,)).copy()

    for sc in SCENARIOS:
        inp = sc.inputs()
        P = run_mex(drv, sc, inp)
        rec = {
            "in_freqRes": inp["freqRes"], "in_TimeDim": inp["TimeDim"],
            "in_pw": inp["pw"], "in_source": inp["source"],
        }
        for f, a in inp["mats"].items():
            rec[f"in_mat{f}"] = a
        if inp["probes"] is not None:
            rec["in_probes"] = inp["probes"]
        ijk = int(np.prod(sc.dims))
        rng = np.random.default_rng(1234)
        smp_idx = np.sort(rng.choice(ijk, size=512, replace=False)).astype(np.int64)
        rec["smp_index"] = smp_idx
        # E through the public OutputVis op must equal the internal arrays
        for flag, name in ((1, "Ex"), (2, "Ey"), (3, "Ez")):
            vis = drv("OutputVis", P, np.uint32(ijk), np.int32(flag))
            assert np.array_equal(vis, ref_array(P, name))
        for name in FIELD_NAMES + PSI_NAMES + COEF_NAMES:
            a = ref_array(P, name)
            rec[f"sha_{name}"] = sha(a)
            rec[f"norm_{name}"] = np.float64(np.linalg.norm(a.astype(np.float64)))
            if name in FIELD_NAMES + COEF_NAMES:
                rec[f"smp_{name}"] = a[smp_idx]
        if sc.mode:
            for name in TABLE_NAMES:
                a = ref_array(P, name)
                rec[f"sha_{name}"] = sha(a)
                rec[f"norm_{name}"] = np.float64(np.linalg.norm(a.astype(np.float64)))
        for name in ("b_E", "c_E", "b_H", "c_H"):
            rec[name] = ref_array(P, name)
        rec["den_ex"] = ref_array(P, "den_ex")[: sc.dims[0]]
        rec["den_hx"] = ref_array(P, "den_hx")[: sc.dims[0]]
        rec["Chh"] = np.float32(drv.lib.ref_scalar(int(P[0]), b"Chh"))
        rec["Che"] = np.float32(drv.lib.ref_scalar(int(P[0]), b"Che"))
        drv("DeleteSimulation", P)
        path = os.path.join(OUT, f"{sc.name}.npz")
        np.savez_compressed(path, **rec)
        print(f"{sc.name}: {os.path.getsize(path) / 1024:.1f} KiB  "
              f"|Ez|={rec['norm_Ez']:.6e} |Hy|={rec['norm_Hy']:.6e}")


if __name__ == "__main__":
    main()
