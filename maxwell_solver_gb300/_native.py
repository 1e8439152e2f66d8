"""ctypes binding of libfdtd_gb300.so (the C ABI of include/fdtd_gb300.h).

The library is built in-tree (maxwell_solver_gb300/build.py).  There is no
CPU fallback: if the library cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .build import LIB

_lock = threading.Lock()
_lib = None

P = ctypes.c_void_p
U64 = ctypes.c_uint64
I32 = ctypes.c_int32
SZ = ctypes.c_size_t


class FdtdParams(ctypes.Structure):
    _fields_ = [("pml", I32), ("tfsf_width", I32), ("poly_m", ctypes.c_double),
                ("alpha_m", ctypes.c_double), ("alpha_max", ctypes.c_double),
                ("kappa_max", ctypes.c_double), ("sig_factor", ctypes.c_double),
                ("r0", ctypes.c_double)]


class FdtdCurrent(ctypes.Structure):
    _fields_ = [("mode", I32), ("box", I32 * 6)]


class FdtdShape(ctypes.Structure):
    _fields_ = [("kind", I32), ("eps_r", ctypes.c_float), ("sigma", ctypes.c_float),
                ("reserved", I32), ("g", ctypes.c_double * 6)]


def shapes_array(rows):
    """ctypes array of FdtdShape from rows [kind, eps_r, sigma, g0..g5]."""
    rows = [list(r) for r in rows]
    arr = (FdtdShape * max(1, len(rows)))()
    for n, r in enumerate(rows):
        g = [float(x) for x in r[3:9]] + [0.0] * (9 - max(len(r), 3))
        arr[n] = FdtdShape(int(r[0]), float(r[1]), float(r[2]), 0, (ctypes.c_double * 6)(*g[:6]))
    return arr


class FdtdRequest(ctypes.Structure):
    _fields_ = [("I", I32), ("J", I32), ("K", I32), ("steps", I32),
                ("fctr", ctypes.c_float), ("delX", ctypes.c_float), ("delT", ctypes.c_float),
                ("params", FdtdParams), ("tfsf_mode", I32), ("rate", ctypes.c_float),
                ("waveform", ctypes.POINTER(ctypes.c_float)),
                ("bg_eps_r", ctypes.c_float), ("bg_sigma", ctypes.c_float),
                ("shapes", ctypes.POINTER(FdtdShape)), ("n_shapes", I32),
                ("n_probes", I32), ("probes", ctypes.POINTER(I32)), ("out_field", I32),
                ("theta", ctypes.c_double), ("phi", ctypes.c_double), ("psi", ctypes.c_double)]


class FdtdServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_uint64), ("max_active", I32), ("round_steps", I32),
                ("one_at_a_time", I32), ("fill_cells", ctypes.c_int64),
                ("solo_cells", ctypes.c_int64), ("policy", I32)]


class FdtdRequestInfo(ctypes.Structure):
    _fields_ = [("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("finish_s", ctypes.c_double), ("device_bytes", ctypes.c_uint64),
                ("status", I32), ("steps", I32), ("message", ctypes.c_char * 128)]


class FdtdServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("cell_steps", ctypes.c_uint64),
                ("peak_reserved_bytes", ctypes.c_uint64), ("peak_active", I32),
                ("queued", I32), ("active", I32), ("elapsed_s", ctypes.c_double),
                ("latency_p50_s", ctypes.c_double), ("latency_p90_s", ctypes.c_double),
                ("latency_p99_s", ctypes.c_double), ("latency_mean_s", ctypes.c_double),
                ("solves_per_s", ctypes.c_double), ("hbm_budget", ctypes.c_uint64),
                ("cancelled", ctypes.c_uint64)]


class FdtdInfo(ctypes.Structure):
    _fields_ = [("I", I32), ("J", I32), ("K", I32), ("T", I32), ("num_ant", I32),
                ("pml", I32), ("size_1d", I32), ("i0", I32), ("i1", I32), ("j0", I32),
                ("j1", I32), ("k0", I32), ("k1", I32), ("coef_mode", I32),
                ("num_materials", I32), ("device_bytes", ctypes.c_uint64),
                ("Chh", ctypes.c_float), ("Che", ctypes.c_float),
                ("zchunk_h", I32), ("zchunk_e", I32), ("hcoef_mode", I32), ("fused", I32),
                ("zchunk_f", I32), ("tile_h", I32), ("tile_e", I32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "fdtd_default_params": (FdtdParams, []),
    "fdtd_set_params": (ctypes.c_int, [U64, ctypes.POINTER(FdtdParams)]),
    "fdtd_create": (ctypes.c_int, [ctypes.POINTER(U64)]),
    "fdtd_destroy": (ctypes.c_int, [U64]),
    "fdtd_set_const": (ctypes.c_int, [U64, P, P]),
    "fdtd_set_source": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_update_source": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_update_material": (ctypes.c_int, [U64, I32, P, SZ]),
    "fdtd_set_incidence": (ctypes.c_int, [U64, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double]),
    "fdtd_set_shapes": (ctypes.c_int, [U64, ctypes.c_float, ctypes.c_float,
                                       ctypes.POINTER(FdtdShape), I32]),
    "fdtd_create_mu": (ctypes.c_int, [U64, P, P, P, SZ]),
    "fdtd_set_magnetic": (ctypes.c_int, [U64, P, P, P, P, P, P, SZ]),
    "fdtd_set_antenna_locations": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_ready_simulation": (ctypes.c_int, [U64]),
    "fdtd_init_1d": (ctypes.c_int, [U64, ctypes.c_float, P, SZ]),
    "fdtd_update_cuda": (ctypes.c_int, [U64]),
    "fdtd_reset_field_all": (ctypes.c_int, [U64]),
    "fdtd_update_h_all": (ctypes.c_int, [U64]),
    "fdtd_update_e_all": (ctypes.c_int, [U64]),
    "fdtd_update_h_pml": (ctypes.c_int, [U64]),
    "fdtd_update_e_pml": (ctypes.c_int, [U64]),
    "fdtd_update_h_planewave": (ctypes.c_int, [U64, I32, I32]),
    "fdtd_update_e_planewave": (ctypes.c_int, [U64, I32, I32]),
    "fdtd_add_currents": (ctypes.c_int, [U64, I32, I32, P]),
    "fdtd_output_ant": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_output_vis": (ctypes.c_int, [U64, P, SZ, I32]),
    "fdtd_step_n": (ctypes.c_int, [U64, I32, I32, I32, ctypes.POINTER(FdtdCurrent)]),
    "fdtd_output_probes": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_synchronize": (ctypes.c_int, [U64]),
    "fdtd_get_info": (ctypes.c_int, [U64, ctypes.POINTER(FdtdInfo)]),
    "fdtd_get_table": (ctypes.c_int, [U64, I32, P, SZ]),
    "fdtd_checkpoint_size": (ctypes.c_int, [U64, ctypes.POINTER(SZ)]),
    "fdtd_checkpoint_save": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_checkpoint_load": (ctypes.c_int, [U64, P, SZ]),
    "fdtd_event_record": (ctypes.c_int, [U64, I32]),
    "fdtd_event_elapsed_ms": (ctypes.c_int, [U64, I32, I32, ctypes.POINTER(ctypes.c_float)]),
    "fdtd_profile_steps": (ctypes.c_int, [U64, I32, I32, I32, ctypes.POINTER(FdtdCurrent),
                                          ctypes.POINTER(ctypes.c_float * 6)]),
    "fdtd_set_device": (ctypes.c_int, [I32]),
    "fdtd_index_coefficients_static": (ctypes.c_int, [ctypes.POINTER(P), I32, I32, I32, I32, P,
                                                      P, I32, ctypes.POINTER(I32), P]),
    "fdtd_batch_create": (ctypes.c_int, [ctypes.POINTER(U64)]),
    "fdtd_batch_destroy": (ctypes.c_int, [U64]),
    "fdtd_batch_add": (ctypes.c_int, [U64, U64, I32, I32, I32, ctypes.POINTER(FdtdCurrent)]),
    "fdtd_batch_step": (ctypes.c_int, [U64, I32, ctypes.POINTER(I32)]),
    "fdtd_batch_get_zrun": (ctypes.c_int, [U64, ctypes.POINTER(I32)]),
    "fdtd_batch_run": (ctypes.c_int, [U64]),
    "fdtd_batch_clear": (ctypes.c_int, [U64]),
    "fdtd_batch_progress": (ctypes.c_int, [U64, U64, ctypes.POINTER(I32)]),
    "fdtd_batch_remove": (ctypes.c_int, [U64, U64]),
    "fdtd_batch_status": (ctypes.c_int, [U64]),
    "fdtd_server_create": (ctypes.c_int, [ctypes.POINTER(U64), ctypes.POINTER(FdtdServerConfig)]),
    "fdtd_server_destroy": (ctypes.c_int, [U64]),
    "fdtd_server_submit": (ctypes.c_int, [U64, ctypes.POINTER(FdtdRequest),
                                          ctypes.POINTER(ctypes.c_uint64)]),
    "fdtd_server_wait": (ctypes.c_int, [U64, ctypes.c_uint64, ctypes.c_double]),
    "fdtd_server_result": (ctypes.c_int, [U64, ctypes.c_uint64, P, SZ, P, SZ,
                                          ctypes.POINTER(FdtdRequestInfo)]),
    "fdtd_server_drain": (ctypes.c_int, [U64]),
    "fdtd_server_get_stats": (ctypes.c_int, [U64, ctypes.POINTER(FdtdServerStats)]),
    "fdtd_server_cancel": (ctypes.c_int, [U64, ctypes.c_uint64]),
    "fdtd_inject_fault": (ctypes.c_int, [I32, I32]),
    "fdtd_inject_device_error": (ctypes.c_int, [U64, I32]),
    "fdtd_estimate_device_bytes": (ctypes.c_int, [I32, I32, I32, I32, I32, I32,
                                                  ctypes.POINTER(ctypes.c_uint64)]),
    "fdtd_division_plan": (ctypes.c_int, [ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "fdtd_check_division": (ctypes.c_int, [ctypes.c_float, ctypes.POINTER(ctypes.c_uint64)]),
    "fdtd_check_bounded_wait": (ctypes.c_int, [ctypes.POINTER(I32), ctypes.POINTER(I32),
                                               ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_double)]),
    "fdtd_launch_count": (ctypes.c_uint64, []),
    "fdtd_last_error": (ctypes.c_char_p, []),
    "fdtd_create_signal": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, SZ, P, ctypes.POINTER(ctypes.c_double)]),
}


def lib_path() -> str:
    return os.environ.get("FDTD_GB300_LIB", LIB)


def load():
    """Loads (never builds) the native library; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                raise ImportError(
                    f"libfdtd_gb300.so not found at {path}: run "
                    "`python -c 'import __graft_entry__ as g; g.build()'` "
                    "(there is no CPU fallback)")
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


STATUS_NAMES = {
    0: "FDTD_OK", 1: "FDTD_ERR_INVALID_HANDLE", 2: "FDTD_ERR_INVALID_ARG",
    3: "FDTD_ERR_STATE", 4: "FDTD_ERR_ALREADY_INITIALIZED", 5: "FDTD_ERR_CUDA",
    6: "FDTD_ERR_OOM", 7: "FDTD_ERR_UNSUPPORTED", 8: "FDTD_ERR_CANCELLED",
}
