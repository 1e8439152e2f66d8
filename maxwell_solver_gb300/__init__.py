"""GB300-native (sm_103a) FDTD step loop with the reference's simFDTD interface.

The compute is libfdtd_gb300.so (C host + hand-written CUDA kernels, C ABI in
include/fdtd_gb300.h); this package binds it with ctypes.  No CPU fallback.
"""
from .simfdtd import SimFDTDError, create_signal, get_table, info, launch_count, simFDTD

__all__ = ["simFDTD", "SimFDTDError", "create_signal", "info", "get_table", "launch_count"]
