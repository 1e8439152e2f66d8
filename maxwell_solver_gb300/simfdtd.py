"""Python mirror of the reference's MEX dispatcher (src/simFDTD.cu:19-187).

``simFDTD(op, P, *args)`` takes the same case-insensitive op strings and
argument meaning as the MATLAB entry point, so a port of highfrequency.m or
GICsimulation.m reads line for line:

    P = simFDTD('CreateSimulation')
    simFDTD('SetConst', P, np.float32([fctr, delX, delT]), np.int32([T, I, J, K, 0]))
    ...
    for n in range(T):
        simFDTD('UpdateH_All', P)
        simFDTD('UpdateH_PlaneWave', P, np.int32([n, 3]))
        ...

Errors raise :class:`SimFDTDError` carrying the reference's identifiers
(simFDTD:InvalidInput, simFDTD:UnknownOperation, simFDTD:AlreadyInitialized)
or the ones this library adds for cases the reference leaves undefined.
Array arguments are flattened in MATLAB (column-major, x fastest) order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

_IDS = {
    1: "simFDTD:InvalidHandle", 2: "simFDTD:InvalidInput", 3: "simFDTD:InvalidState",
    4: "simFDTD:AlreadyInitialized", 5: "simFDTD:CudaError", 6: "simFDTD:OutOfMemory",
    7: "simFDTD:Unsupported",
}


class SimFDTDError(RuntimeError):
    def __init__(self, identifier: str, message: str, status: int = 0):
        super().__init__(f"{identifier}: {message}")
        self.identifier = identifier
        self.message = message
        self.status = status


def _check(rc: int):
    if rc != 0:
        lib = _native.load()
        msg = (lib.fdtd_last_error() or b"").decode(errors="replace")
        raise SimFDTDError(_IDS.get(rc, "simFDTD:Failed"), msg, rc)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel(order="F"))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _handle(P) -> int:
    return int(np.asarray(P, dtype=np.uint64).ravel()[0])


def simFDTD(op: str, *args):  # noqa: N802 - mirrors the MATLAB entry point
    lib = _native.load()
    if not isinstance(op, str):
        raise SimFDTDError("simFDTD:InvalidInput", "At least one input required: operation string.")
    o = op.lower()
    if o == "createsimulation":
        h = ctypes.c_uint64(0)
        _check(lib.fdtd_create(ctypes.byref(h)))
        return np.array([h.value], dtype=np.uint64)
    if len(args) < 1:
        raise SimFDTDError("simFDTD:InvalidInput", "Simulation pointer required for this operation.")
    P = _handle(args[0])
    a = args[1:]

    def need(n, msg):
        if len(a) < n:
            raise SimFDTDError("simFDTD:InvalidInput", msg)

    if o == "deletesimulation":
        _check(lib.fdtd_destroy(P))
    elif o == "updatee_all":
        _check(lib.fdtd_update_e_all(P))
    elif o == "updateh_all":
        _check(lib.fdtd_update_h_all(P))
    elif o == "updatee_pml":
        _check(lib.fdtd_update_e_pml(P))
    elif o == "updateh_pml":
        _check(lib.fdtd_update_h_pml(P))
    elif o == "updatecuda":
        _check(lib.fdtd_update_cuda(P))
    elif o == "addcurrents":
        need(2, "time and indices required.")
        t, box = _i32(a[0]), _i32(a[1])
        if t.size < 2 or box.size < 6:
            raise SimFDTDError("simFDTD:InvalidInput", "time and indices required.")
        _check(lib.fdtd_add_currents(P, int(t[0]), int(t[1]), _ptr(box)))
    elif o == "readysimulation":
        _check(lib.fdtd_ready_simulation(P))
    elif o == "resetfieldall":
        _check(lib.fdtd_reset_field_all(P))
    elif o in ("updatee_planewave", "updateh_planewave"):
        need(1, "time required.")
        t = _i32(a[0])
        if t.size < 2:
            raise SimFDTDError("simFDTD:InvalidInput", "time required.")
        fn = lib.fdtd_update_e_planewave if o[6] == "e" else lib.fdtd_update_h_planewave
        _check(fn(P, int(t[0]), int(t[1])))
    elif o == "setconst":
        need(2, "freqRes and TimeDim required.")
        fr, td = _f32(a[0]), _i32(a[1])
        if fr.size < 3 or td.size < 5:
            raise SimFDTDError("simFDTD:InvalidInput", "freqRes and TimeDim required.")
        _check(lib.fdtd_set_const(P, _ptr(fr), _ptr(td)))
    elif o == "setsource":
        need(1, "SourceIn required.")
        src = _f32(a[0])
        fn = lib.fdtd_update_source if len(a) > 1 else lib.fdtd_set_source
        _check(fn(P, _ptr(src), src.size))
    elif o == "setantennalocations":
        need(1, "Locations required.")
        loc = _i32(a[0])
        _check(lib.fdtd_set_antenna_locations(P, _ptr(loc), loc.size))
    elif o == "createmu":
        need(3, "mu_x, mu_y, mu_z required.")
        mx, my, mz = _f32(a[0]), _f32(a[1]), _f32(a[2])
        _check(lib.fdtd_create_mu(P, _ptr(mx), _ptr(my), _ptr(mz), min(mx.size, my.size, mz.size)))
    elif o == "setmagnetic":
        if len(a) not in (3, 6):
            raise SimFDTDError("simFDTD:InvalidInput", "mu_x, mu_y, mu_z [, sm_x, sm_y, sm_z] required.")
        v = [_f32(x) for x in a]
        n = min(x.size for x in v)
        ptrs = [_ptr(x) for x in v] + [None] * (6 - len(v))
        _check(lib.fdtd_set_magnetic(P, *ptrs, n))
    elif o == "init1d":
        need(2, "rate and PW_source required.")
        rate, pw = _f32(a[0]), _f32(a[1])
        _check(lib.fdtd_init_1d(P, float(rate[0]), _ptr(pw), pw.size))
    elif o == "updatematerial":
        need(2, "flag, values required.")
        flag, v = _i32(a[0]), _f32(a[1])
        _check(lib.fdtd_update_material(P, int(flag[0]), _ptr(v), v.size))
    elif o == "setincidence":
        need(1, "[theta phi psi] required.")
        v = np.asarray(a[0], dtype=np.float64).ravel()
        if v.size < 3:
            raise SimFDTDError("simFDTD:InvalidInput", "[theta phi psi] required.")
        _check(lib.fdtd_set_incidence(P, float(v[0]), float(v[1]), float(v[2])))
    elif o == "setshapes":
        # [bg_eps_r bg_sigma], rows [kind eps_r sigma g0 .. g5] (FDTD_SHAPE_*)
        need(2, "background and shapes required.")
        bg = _f32(a[0])
        rows = np.asarray(a[1], dtype=np.float64).reshape(-1, 9) if np.size(a[1]) else \
            np.zeros((0, 9))
        if bg.size < 2:
            raise SimFDTDError("simFDTD:InvalidInput", "background and shapes required.")
        arr = _native.shapes_array(rows)
        _check(lib.fdtd_set_shapes(P, float(bg[0]), float(bg[1]), arr, len(rows)))
    elif o == "outputant":
        need(1, "OutAntSize required.")
        n = int(np.asarray(a[0]).ravel()[0])
        out = np.zeros(n, dtype=np.float32)
        rc = lib.fdtd_output_ant(P, _ptr(out), n)
        if rc != 3:  # not initialised: the reference prints and returns zeros
            _check(rc)
        return out
    elif o == "outputvis":
        need(2, "OutAntSize and flag required.")
        n = int(np.asarray(a[0]).ravel()[0])
        flag = int(_i32(a[1])[0])
        out = np.zeros(n, dtype=np.float32)
        _check(lib.fdtd_output_vis(P, _ptr(out), n, flag))
        return out
    elif o == "outputprobes":
        need(1, "OutSize required.")
        n = int(np.asarray(a[0]).ravel()[0])
        out = np.zeros(n, dtype=np.float32)
        _check(lib.fdtd_output_probes(P, _ptr(out), n))
        return out
    elif o == "stepn":
        need(1, "[first count mode] required.")
        t = _i32(a[0])
        cur = None
        if len(a) > 1:
            c = _i32(a[1])
            if c.size >= 7:
                cur = _native.FdtdCurrent(int(c[0]), (ctypes.c_int32 * 6)(*[int(x) for x in c[1:7]]))
        _check(lib.fdtd_step_n(P, int(t[0]), int(t[1]), int(t[2]) if t.size > 2 else 0,
                               ctypes.byref(cur) if cur is not None else None))
    elif o == "setparams":
        need(1, "params required.")
        v = np.asarray(a[0], dtype=np.float64).ravel()
        pr = lib.fdtd_default_params()
        names = ("pml", "tfsf_width", "poly_m", "alpha_m", "alpha_max", "kappa_max",
                 "sig_factor", "r0")
        for i, nm in enumerate(names[: v.size]):
            setattr(pr, nm, int(v[i]) if i < 2 else float(v[i]))
        _check(lib.fdtd_set_params(P, ctypes.byref(pr)))
    elif o == "synchronize":
        _check(lib.fdtd_synchronize(P))
    elif o == "savecheckpoint":
        n = ctypes.c_size_t(0)
        _check(lib.fdtd_checkpoint_size(P, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.uint8)
        _check(lib.fdtd_checkpoint_save(P, _ptr(out), out.size))
        return out
    elif o == "loadcheckpoint":
        need(1, "checkpoint required.")
        buf = np.ascontiguousarray(a[0], dtype=np.uint8)
        _check(lib.fdtd_checkpoint_load(P, _ptr(buf), buf.size))
    else:
        raise SimFDTDError("simFDTD:UnknownOperation", f"Unknown operation: {o}")
    return None


def create_signal(fctr, delT, percentage_bw, num_side_lobes, time_steps):
    """FunLib('CreateSignal', ...) (src/cpucode/FunLib.cpp:6-45): returns
    (fmaxx, source) in double precision."""
    lib = _native.load()
    out = np.zeros(int(time_steps), dtype=np.float64)
    fmaxx = ctypes.c_double(0.0)
    _check(lib.fdtd_create_signal(float(fctr), float(delT), float(percentage_bw),
                                  float(num_side_lobes), int(time_steps), _ptr(out),
                                  ctypes.byref(fmaxx)))
    return fmaxx.value, out


def info(P) -> dict:
    lib = _native.load()
    inf = _native.FdtdInfo()
    _check(lib.fdtd_get_info(_handle(P), ctypes.byref(inf)))
    return {name: getattr(inf, name) for name, _ in inf._fields_}


def get_table(P, which: str) -> np.ndarray:
    lib = _native.load()
    idx = ("b_E", "c_E", "b_H", "c_H", "den_ex", "den_hx", "materials").index(which)
    inf = info(P)
    n = 2 * inf["pml"] if idx < 4 else (inf["I"] if idx < 6 else 6 * inf["num_materials"])
    out = np.zeros(n, dtype=np.float32)
    _check(lib.fdtd_get_table(_handle(P), idx, _ptr(out), n))
    return out


def launch_count() -> int:
    return int(_native.load().fdtd_launch_count())
