"""Batched execution: many simulations of different sizes advanced together.

    b = Batch()
    b.add(P1, first=0, count=500, mode=3)
    b.add(P2, first=0, count=800, mode=1, current=(1, [i0, i1, j0, j1, k0, k1]))
    b.run()          # or repeated b.step(n) with b.add() in between

Each member is an ordinary handle from simFDTD('CreateSimulation') set up
with the usual ops; after the batch its results are read with OutputVis /
OutputProbes as usual, and they equal running the handle alone bit for bit.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .simfdtd import _check, _handle


class Batch:
    def __init__(self):
        self._lib = _native.load()
        h = ctypes.c_uint64(0)
        _check(self._lib.fdtd_batch_create(ctypes.byref(h)))
        self.handle = h.value

    def add(self, P, first: int, count: int, mode: int = 0, current=None):
        cur = None
        if current is not None:
            cmode, box = current
            cur = _native.FdtdCurrent(int(cmode), (ctypes.c_int32 * 6)(*[int(x) for x in box]))
        _check(self._lib.fdtd_batch_add(self.handle, _handle(P), int(first), int(count),
                                        int(mode), ctypes.byref(cur) if cur else None))

    def step(self, max_steps: int) -> int:
        left = ctypes.c_int32(0)
        _check(self._lib.fdtd_batch_step(self.handle, int(max_steps), ctypes.byref(left)))
        return left.value

    def run(self):
        _check(self._lib.fdtd_batch_run(self.handle))

    def clear(self):
        _check(self._lib.fdtd_batch_clear(self.handle))

    def progress(self, P) -> int:
        d = ctypes.c_int32(0)
        _check(self._lib.fdtd_batch_progress(self.handle, _handle(P), ctypes.byref(d)))
        return d.value

    @property
    def zrun(self) -> int:
        """z-planes per batched work item (0 until the batch has measured it)."""
        z = ctypes.c_int32(0)
        _check(self._lib.fdtd_batch_get_zrun(self.handle, ctypes.byref(z)))
        return z.value

    def close(self):
        if self.handle:
            _check(self._lib.fdtd_batch_destroy(self.handle))
            self.handle = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def as_int_list(a):
    return [int(x) for x in np.asarray(a).ravel()]
