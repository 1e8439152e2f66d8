"""ctypes driver for mexFunction implementations linked with tests/mexstub.

MATLAB is absent, so tests call a library's mexFunction the way a MATLAB
script would (``drv('UpdateH_PlaneWave', P, np.int32([n, 3]))``): arguments
become stub mxArrays of the matching class, errors raised through
mexErrMsgIdAndTxt come back as :class:`MexError` with their identifier.
"""
from __future__ import annotations

import ctypes

import numpy as np

MX_CHAR, MX_DOUBLE, MX_SINGLE, MX_INT32, MX_UINT32, MX_UINT64 = 4, 6, 7, 12, 13, 15
MX_UINT8 = 9
_CLASS_OF = {
    np.dtype(np.uint8): MX_UINT8,
    np.dtype(np.float64): MX_DOUBLE,
    np.dtype(np.float32): MX_SINGLE,
    np.dtype(np.int32): MX_INT32,
    np.dtype(np.uint32): MX_UINT32,
    np.dtype(np.uint64): MX_UINT64,
}
_DTYPE_OF = {v: k for k, v in _CLASS_OF.items()}


class MexError(RuntimeError):
    def __init__(self, ident: str, msg: str):
        super().__init__(f"{ident}: {msg}")
        self.identifier = ident
        self.message = msg


class MexDriver:
    def __init__(self, lib_path: str, entry: str = "mexFunction"):
        self.lib = ctypes.CDLL(lib_path)
        L = self.lib
        P = ctypes.c_void_p
        L.mxCreateString.restype = P
        L.mxCreateString.argtypes = [ctypes.c_char_p]
        L.mexstub_numeric.restype = P
        L.mexstub_numeric.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, P]
        L.mxDestroyArray.argtypes = [P]
        L.mxGetData.restype = P
        L.mxGetData.argtypes = [P]
        L.mxGetM.restype = ctypes.c_size_t
        L.mxGetM.argtypes = [P]
        L.mxGetN.restype = ctypes.c_size_t
        L.mxGetN.argtypes = [P]
        L.mxGetClassID.restype = ctypes.c_int
        L.mxGetClassID.argtypes = [P]
        L.mexstub_printed.restype = ctypes.c_char_p
        L.mexstub_call.restype = ctypes.c_int
        L.mexstub_call.argtypes = [P, ctypes.c_int, P, ctypes.c_int, P,
                                   ctypes.c_char_p, ctypes.c_size_t,
                                   ctypes.c_char_p, ctypes.c_size_t]
        self.fn = ctypes.cast(getattr(L, entry), P)

    def _to_mx(self, a):
        if isinstance(a, str):
            return self.lib.mxCreateString(a.encode())
        arr = np.asarray(a)
        if arr.dtype not in _CLASS_OF:
            raise TypeError(f"unsupported argument dtype {arr.dtype}")
        arr = np.ascontiguousarray(arr.ravel(order="F"))
        return self.lib.mexstub_numeric(_CLASS_OF[arr.dtype], 1, arr.size,
                                        arr.ctypes.data_as(ctypes.c_void_p))

    def _from_mx(self, m):
        cls = self.lib.mxGetClassID(m)
        n = self.lib.mxGetM(m) * self.lib.mxGetN(m)
        dt = _DTYPE_OF.get(cls)
        if dt is None:
            return None
        buf = (ctypes.c_byte * (n * dt.itemsize)).from_address(self.lib.mxGetData(m)) if n else b""
        return np.frombuffer(bytes(buf), dtype=dt).copy()

    @property
    def printed(self) -> str:
        return self.lib.mexstub_printed().decode(errors="replace")

    def __call__(self, *args, nlhs: int = 1):
        prhs = [self._to_mx(a) for a in args]
        arr_in = (ctypes.c_void_p * max(1, len(prhs)))(*prhs)
        arr_out = (ctypes.c_void_p * max(1, nlhs))()
        eid = ctypes.create_string_buffer(128)
        emsg = ctypes.create_string_buffer(512)
        try:
            rc = self.lib.mexstub_call(self.fn, nlhs, arr_out, len(prhs), arr_in,
                                       eid, 128, emsg, 512)
            if rc:
                raise MexError(eid.value.decode(), emsg.value.decode())
            outs = []
            for i in range(nlhs):
                if arr_out[i]:
                    outs.append(self._from_mx(arr_out[i]))
                    self.lib.mxDestroyArray(arr_out[i])
                else:
                    outs.append(None)
        finally:
            for m in prhs:
                self.lib.mxDestroyArray(m)
        return outs[0] if nlhs == 1 else tuple(outs)
