"""A grid of more than 2^31 cells (1300^3 = 2.197e9): every cell index in
the kernels and the host is 64-bit.  Until a wave reaches the CPML, the
fields near a source do not depend on how far away the boundaries are, so a
current source with a dielectric sphere beside it, in the middle of the
huge grid and of a 128^3 grid, must give bit-identical probe records for
the first 40 steps (the CPML is 50 cells away in the small grid)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PML, STEPS = 10, 40
OFFS = [(0, 0, 0), (3, 0, 0), (0, -4, 2), (-6, 5, -3), (9, 9, 9), (-12, 0, 7)]


def _record(n):
    from maxwell_solver_gb300.workloads import SHAPE_SPHERE
    from maxwell_solver_gb300 import simFDTD

    c = n // 2
    dx = 1e-3
    dt = 0.99 * dx / (math.sqrt(3) * 299792458.0)
    P = simFDTD("CreateSimulation")
    simFDTD("SetParams", P, np.float64([PML, PML + 5, 3, 1, 0.08, 1, 0.8, 0]))
    simFDTD("SetConst", P, np.float32([30e9, dx, dt]), np.int32([STEPS, n, n, n, len(OFFS)]))
    t = np.arange(STEPS, dtype=np.float64)
    simFDTD("SetSource", P, np.exp(-((t - 12) / 4) ** 2).astype(np.float32))
    rows = np.array([[SHAPE_SPHERE, 4.0, 0.01, c + 4.5, c + 0.5, c - 2.5, 3.0, 0, 0]])
    simFDTD("SetShapes", P, np.float32([1.0, 0.0]), rows)
    loc = np.array([[c + a - PML, c + b - PML, c + d - PML] for a, b, d in OFFS], np.int32)
    simFDTD("SetAntennaLocations", P, np.asfortranarray(loc))
    simFDTD("ReadySimulation", P)
    simFDTD("StepN", P, np.int32([0, STEPS, 0]), np.int32([3, c, c, c, c, c, c]))
    rec = simFDTD("OutputProbes", P, np.uint32(STEPS * len(OFFS) * 6))
    simFDTD("DeleteSimulation", P)
    return rec


def test_grid_beyond_2_31_cells(monkeypatch):
    monkeypatch.setenv("FDTD_AUTOTUNE", "0")
    big = _record(1300)
    small = _record(128)
    assert 1300 ** 3 > 2 ** 31
    assert np.abs(small).max() > 0
    np.testing.assert_array_equal(big, small)
