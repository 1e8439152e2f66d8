"""Generates tests/golden/funlib_signal.npz from the reference itself.

Drives the reference's source-waveform MEX file (src/cpucode/FunLib.cpp,
'CreateSignal' -> [fmaxx, source]), built for the host by
oracle/funlib_build.sh against tests/mexstub, over a few argument sets, and
stores the arguments and both outputs (float64).  The set covers the
configurations' centre frequencies, a time step count that ends inside the
pulse (2*tto > T), one whose window spans many pulses, and a centre where
the sinc argument passes through zero.

Needs the reference sources ($MAXWELL_REF, or the path given as the first
argument); the committed .npz is what the tests read.
Usage:  python tests/golden/make_funlib_golden.py [reference_root]
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from mexstub.mexdrv import MexDriver  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "funlib_signal.npz")
C0 = 299792458.0

# (fctr, delT, PercentageBW, NumOfSidLobes, timeSteps)
CASES = [
    (30e9, 0.99 * 1e-3 / (math.sqrt(3) * C0), 0.5, 3.0, 500),
    (1e9, 0.99 * 5e-3 / (math.sqrt(3) * C0), 1.0, 2.0, 4000),
    (10e9, 0.99 * 2e-3 / (math.sqrt(3) * C0), 0.25, 6.0, 120),
    (60e9, 0.99 * 1e-3 / (math.sqrt(3) * C0), 1.5, 1.0, 1500),
    (20e9, 1.25e-12, 0.8, 4.0, 3000),
]


def main():
    lib = oracle.build_reference_funlib(sys.argv[1] if len(sys.argv) > 1 else None)
    if lib is None:
        raise SystemExit("reference sources not found; cannot regenerate the waveform vectors")
    drv = MexDriver(lib, "mexFunction")
    out = {"args": np.array(CASES, dtype=np.float64)}
    for c, (fctr, dt, bw, lobes, T) in enumerate(CASES):
        fmaxx, src = drv("CreateSignal", np.float64(fctr), np.float64(dt), np.float64(bw),
                         np.float64(lobes), np.float64(T), nlhs=2)
        out[f"fmaxx_{c}"] = np.float64(fmaxx[0])
        out[f"source_{c}"] = src.astype(np.float64)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {len(CASES)} cases")


if __name__ == "__main__":
    main()
