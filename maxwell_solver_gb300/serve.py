"""Serving: solve requests admitted against a device-memory budget and run
with continuous batching by the library's C request loop (fdtd_server_* in
include/fdtd_gb300.h).

    srv = Server(hbm_budget=120 << 30)
    t = srv.submit(spec)              # a workloads.GridSpec (or submit_request)
    out = srv.result(t)               # waits; {'probes', 'field', 'info'}
    srv.stats()                       # solves/s, p50/p90/p99 latency, ...
    srv.close()

Server(one_at_a_time=True) runs the same requests as a plain FIFO queue
through fdtd_step_n, one solve on the device at a time.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .simfdtd import SimFDTDError, _check
from .workloads import GridSpec, grid_probes, grid_shapes, grid_source


class Server:
    def __init__(self, hbm_budget: int = 120 << 30, max_active: int = 0, round_steps: int = 0,
                 one_at_a_time: bool = False, fill_cells: int = 0, solo_cells: int = 0,
                 policy: str = "srpt"):
        self._lib = _native.load()
        pol = {"srpt": 0, "hrrn": 1, "bounded": 2, "deadline": 3}[policy]
        cfg = _native.FdtdServerConfig(int(hbm_budget), int(max_active), int(round_steps),
                                       int(bool(one_at_a_time)), int(fill_cells), int(solo_cells),
                                       pol)
        h = ctypes.c_uint64(0)
        _check(self._lib.fdtd_server_create(ctypes.byref(h), ctypes.byref(cfg)))
        self.handle = h.value
        self._shape = {}  # ticket -> (steps, n_probes, cells, out_field)

    # ------------------------------------------------------------ requests
    def submit_request(self, dims, steps, fctr, delX, delT, pml, tfsf_mode, waveform,
                       shapes=(), bg=(1.0, 0.0), probes=None, out_field=0, rate=1.0,
                       tfsf_width=None, angles=(0.0, 0.0, 0.0)) -> int:
        I, J, K = (int(x) for x in dims)
        prm = self._lib.fdtd_default_params()
        prm.pml = int(pml)
        prm.tfsf_width = int(pml + 5 if tfsf_width is None else tfsf_width)
        wf = np.ascontiguousarray(waveform, dtype=np.float32)
        sh = _native.shapes_array(list(shapes))
        pr = (np.asfortranarray(probes, dtype=np.int32) if probes is not None
              else np.zeros((0, 3), dtype=np.int32, order="F"))
        req = _native.FdtdRequest()
        req.I, req.J, req.K, req.steps = I, J, K, int(steps)
        req.fctr, req.delX, req.delT = float(fctr), float(delX), float(delT)
        req.params = prm
        req.tfsf_mode = int(tfsf_mode)
        req.rate = float(rate)
        req.waveform = wf.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        req.bg_eps_r, req.bg_sigma = float(bg[0]), float(bg[1])
        req.shapes = sh
        req.n_shapes = len(shapes)
        req.n_probes = int(pr.shape[0])
        req.probes = pr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        req.out_field = int(out_field)
        req.theta, req.phi, req.psi = (float(a) for a in angles)
        t = ctypes.c_uint64(0)
        _check(self._lib.fdtd_server_submit(self.handle, ctypes.byref(req), ctypes.byref(t)))
        self._shape[t.value] = (int(steps), int(pr.shape[0]), I * J * K, int(out_field))
        return t.value

    def submit(self, spec: GridSpec, n_probes: int = 8, out_field: int = 0) -> int:
        bg_e, bg_s, rows = grid_shapes(spec)
        return self.submit_request(spec.dims, spec.steps, spec.fctr, spec.delX, spec.delT,
                                   spec.pml, spec.mode, grid_source(spec), rows, (bg_e, bg_s),
                                   grid_probes(spec, n_probes) if n_probes else None, out_field,
                                   angles=spec.angles if spec.mode == 5 else (0.0, 0.0, 0.0))

    def wait(self, ticket: int, timeout: float | None = None) -> None:
        _check(self._lib.fdtd_server_wait(self.handle, int(ticket),
                                          -1.0 if timeout is None else float(timeout)))

    def result(self, ticket: int, timeout: float | None = None) -> dict:
        self.wait(ticket, timeout)
        steps, n_probes, cells, out_field = self._shape.pop(ticket)
        pr = np.zeros(steps * n_probes * 6, dtype=np.float32)
        fd = np.zeros(cells if out_field else 0, dtype=np.float32)
        info = _native.FdtdRequestInfo()
        rc = self._lib.fdtd_server_result(self.handle, int(ticket),
                                          pr.ctypes.data_as(ctypes.c_void_p), pr.size,
                                          fd.ctypes.data_as(ctypes.c_void_p), fd.size,
                                          ctypes.byref(info))
        out = {"probes": pr, "field": fd if out_field else None,
               "info": {"submit_s": info.submit_s, "admit_s": info.admit_s,
                        "finish_s": info.finish_s, "latency_s": info.finish_s - info.submit_s,
                        "device_bytes": info.device_bytes, "status": info.status,
                        "message": info.message.decode(errors="replace")}}
        if rc:
            name = _native.STATUS_NAMES.get(rc, str(rc))
            raise SimFDTDError("simFDTD:ServeFailed", f"{name}: {out['info']['message']}")
        return out

    def cancel(self, ticket: int) -> int:
        """fdtd_server_cancel: 0 when the request was cancelled (its result
        then raises with FDTD_ERR_CANCELLED), else the status (e.g. 3 when it
        had finished already)."""
        return int(self._lib.fdtd_server_cancel(self.handle, int(ticket)))

    def drain(self) -> None:
        _check(self._lib.fdtd_server_drain(self.handle))

    def stats(self) -> dict:
        st = _native.FdtdServerStats()
        _check(self._lib.fdtd_server_get_stats(self.handle, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in st._fields_}

    def close(self) -> None:
        if self.handle:
            _check(self._lib.fdtd_server_destroy(self.handle))
            self.handle = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def estimate_device_bytes(spec: GridSpec, n_probes: int = 8) -> int:
    """Peak device bytes of one request (fdtd_estimate_device_bytes)."""
    lib = _native.load()
    out = ctypes.c_uint64(0)
    I, J, K = spec.dims
    _check(lib.fdtd_estimate_device_bytes(I, J, K, spec.pml, spec.steps, n_probes,
                                          ctypes.byref(out)))
    return out.value
