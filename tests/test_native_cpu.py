"""CPU-side checks of the native library: it builds, loads, exports every
entry point of include/fdtd_gb300.h, and its host-only paths (argument and
handle validation, the source-waveform generator, the MEX dispatcher's
error identifiers) behave as the reference's interface specifies.  No
compute call is made (there is no GPU here)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from scenarios import create_signal as np_create_signal

HEADER = os.path.join(ROOT, "include", "fdtd_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fdtd_[a-z0-9_]+)\s*\(", text)))


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_header_entry_points_are_exported(native_lib):
    from maxwell_solver_gb300.build import LIB

    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if n not in exported_symbols(LIB)]
    assert not missing, missing


def test_python_binding_covers_header(native_lib):
    from maxwell_solver_gb300._native import SIGNATURES

    assert set(declared_functions()) == set(SIGNATURES)


def test_create_signal_matches_funlib_formula(native_lib):
    from maxwell_solver_gb300 import create_signal

    for args in ((5.5e9, 1.9e-13, 8e9 / 5.5e9, 2, 400), (30e9, 1.9e-12, 0.5, 1, 120)):
        fmaxx, got = create_signal(*args)
        want = np_create_signal(*args)
        assert fmaxx == args[0] * args[2] / 2.0
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)


def test_create_signal_matches_reference_funlib(native_lib):
    """fdtd_create_signal against the reference's own FunLib.cpp
    ('CreateSignal', src/cpucode/FunLib.cpp:6-45), whose outputs for five
    argument sets are in tests/golden/funlib_signal.npz (generated by
    tests/golden/make_funlib_golden.py from the reference built by
    oracle/funlib_build.sh): fmaxx equal, every sample within 1 ulp."""
    from maxwell_solver_gb300 import create_signal

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "funlib_signal.npz"))
    for c, args in enumerate(g["args"]):
        fctr, dt, bw, lobes, steps = (float(v) for v in args)
        fmaxx, got = create_signal(fctr, dt, bw, lobes, int(steps))
        assert fmaxx == float(g[f"fmaxx_{c}"])
        want = g[f"source_{c}"]
        assert got.shape == want.shape
        np.testing.assert_array_max_ulp(got, want, maxulp=1)


def test_invalid_handle_is_rejected(native_lib):
    for fn in ("fdtd_update_h_all", "fdtd_update_e_all", "fdtd_ready_simulation",
               "fdtd_destroy", "fdtd_synchronize"):
        assert getattr(native_lib, fn)(0xDEADBEEF00000001) == 1
    assert native_lib.fdtd_update_h_planewave(0, 0, 3) == 1
    assert b"invalid simulation handle" in native_lib.fdtd_last_error()


def test_default_params_are_reference_constants(native_lib):
    p = native_lib.fdtd_default_params()
    assert (p.pml, p.tfsf_width) == (10, 15)
    assert (p.poly_m, p.alpha_m, p.alpha_max, p.kappa_max, p.sig_factor, p.r0) == \
        (3.0, 1.0, 0.08, 1.0, 0.8, 0.0)


def test_python_dispatcher_errors(native_lib):
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    bogus = np.array([0xDEADBEEF00000001], dtype=np.uint64)
    with pytest.raises(SimFDTDError) as e:
        simFDTD("NoSuchOp", bogus)
    assert e.value.identifier == "simFDTD:UnknownOperation"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("UpdateH_All")
    assert e.value.identifier == "simFDTD:InvalidInput"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("SetConst", bogus)
    assert e.value.identifier == "simFDTD:InvalidInput"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("updateh_all", bogus)  # op strings are case-insensitive
    assert e.value.identifier == "simFDTD:InvalidHandle"


def test_mex_dispatcher_errors(mex):
    from mexstub.mexdrv import MexError

    bogus = np.array([0xDEADBEEF00000001], dtype=np.uint64)
    with pytest.raises(MexError) as e:
        mex("NoSuchOp", bogus)
    assert e.value.identifier == "simFDTD:UnknownOperation"
    assert "nosuchop" in e.value.message
    with pytest.raises(MexError) as e:
        mex(nlhs=1)
    assert e.value.identifier == "simFDTD:InvalidInput"
    with pytest.raises(MexError) as e:
        mex("UpdateE_All")
    assert e.value.identifier == "simFDTD:InvalidInput"
    for op, args in (("AddCurrents", (np.int32([0, 1]),)), ("UpdateH_PlaneWave", ()),
                     ("SetConst", (np.float32([1, 2, 3]),)), ("Init1D", (np.float32([1]),)),
                     ("OutputVis", (np.uint32(8),)), ("CreateMu", ()),
                     ("UpdateMaterial", (np.int32(1),)), ("SetSource", ()),
                     ("SetAntennaLocations", ()), ("OutputAnt", ()),
                     ("SetMagnetic", (np.float32([1]), np.float32([1]))),
                     ("SetIncidence", ()), ("SetShapes", (np.float32([1, 0]),)),
                     ("LoadCheckpoint", ()), ("LoadCheckpoint", (np.float32([1]),)),
                     ("StepN", ())):
        with pytest.raises(MexError) as e:
            mex(op, bogus, *args)
        assert e.value.identifier == "simFDTD:InvalidInput", op
    with pytest.raises(MexError) as e:
        mex("UpdateH_All", bogus)
    assert e.value.identifier == "simFDTD:InvalidHandle"


def _rn32(x):
    """Round an exact rational to the nearest float32 (ties to even)."""
    from fractions import Fraction

    f = np.float32(float(x))  # within one float32 ulp of x
    cands = [f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf))]
    best = min(cands, key=lambda c: (abs(Fraction(float(c)) - x),
                                     int(np.array(c).view(np.uint32)) & 1))
    return best


@pytest.mark.parametrize("dx", [1e-3, 3.7e-4, 1.0, 2.0 / 3.0, 12.5])
def test_division_plan_equals_ieee_quotient(native_lib, dx):
    """The CPML's division by dx is done as a corrected product inside the
    plan's ranges; restated here in exact rational arithmetic, it must give
    RN(a/dx) for numerators drawn across those ranges (the GPU test checks
    every float)."""
    from fractions import Fraction

    out = (ctypes.c_float * 4)()
    assert native_lib.fdtd_division_plan(ctypes.c_float(dx), out) == 0
    y, lo, hi, lo2 = (np.float32(v) for v in out)
    b = np.float32(dx)
    assert y == np.float32(1.0 / float(b))
    # corrected products cover the fields' range down to quotients near the
    # smallest normal float
    assert lo2 <= np.float32(max(1e-38, float(b) * 2.0 ** -123)) and lo <= np.float32(1e-20)
    assert hi >= np.float32(1e30)
    rng = np.random.default_rng(7)
    ex = np.concatenate([rng.uniform(np.log2(float(lo)), np.log2(float(hi)), 300),
                         rng.uniform(np.log2(float(lo2)), np.log2(float(lo)), 100)])
    mags = [np.float32(2.0) ** np.float32(e) for e in ex]
    for a in [np.float32(m * sgn) for m, sgn in zip(mags, rng.choice([-1, 1], len(mags)))]:
        if not (lo2 <= abs(a) < hi):
            continue
        scale = Fraction(2) ** 64 if abs(a) < lo else Fraction(1)
        A, B, Y = Fraction(float(a)) * scale, Fraction(float(b)), Fraction(float(y))
        q0 = _rn32(A * Y)
        r = _rn32(A - B * Fraction(float(q0)))
        q = np.float32(float(Fraction(float(_rn32(Fraction(float(q0)) + Fraction(float(r)) * Y)))
                             / scale))
        assert q == a / b, (a, q, a / b)
