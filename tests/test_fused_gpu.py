"""The fused step (H and E of a step in one pass, fdtd_fused.cu) against
the FP32 oracle, bit for bit: every TF/SF mode (1-4 and oblique 5, whose
face passes and E fix-up run after the pass), spheres in the CPML's
reach, probes, runs through graph replays, single pairs and an odd last
step, through the per-op calls, and with per-cell coefficient arrays
instead of material ids.  FDTD_FUSED=1 makes the handles run the fused
pass whatever the autotuner would choose (checked with fdtd_get_info)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS, PML, W = (64, 56, 60), 8, 13
FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
ANG = (math.radians(55), math.radians(-35), math.radians(70))


@pytest.fixture(autouse=True)
def _force_fused(monkeypatch):
    monkeypatch.setenv("FDTD_FUSED", "1")


def _inputs(steps, seed=5):
    from maxwell_solver_gb300.workloads import SHAPE_SPHERE, rasterize

    I, J, K = DIMS
    dx = 1e-3
    dt = 0.99 * dx / (math.sqrt(3) * 299792458.0)
    rows = [[SHAPE_SPHERE, 4.0, 0.02, 30.5, 27.0, 29.0, 9.5, 0, 0],
            [SHAPE_SPHERE, 2.5, 0.3, 12.0, 14.0, 11.0, 6.0, 0, 0],   # reaches into the CPML
            [SHAPE_SPHERE, 6.0, 0.0, 50.0, 40.0, 45.0, 5.0, 0, 0]]
    eps, sig = rasterize(DIMS, 1.0, 0.0, rows)
    t = np.arange(steps) * np.float32(dt)
    f0, spread = 20e9, 15e-12
    pw = (np.sin(2 * np.pi * f0 * (t - 3 * spread)) *
          np.exp(-((t - 3 * spread) / spread) ** 2)).astype(np.float32)
    rng = np.random.default_rng(seed)
    probes = np.stack([rng.integers(1, d - 2 * PML - 1, 6) for d in DIMS], axis=1).astype(np.int32)
    return dict(fr=np.float32([f0, dx, dt]), td=np.int32([steps, I, J, K, 6]), eps=eps, sig=sig,
                pw=pw, probes=np.asfortranarray(probes), steps=steps)


def _ready(api, inp, mode):
    P = api("CreateSimulation")
    api("SetParams", P, np.float64([PML, W, 3, 1, 0.08, 1, 0.8, 0]))
    api("SetConst", P, inp["fr"], inp["td"])
    api("SetAntennaLocations", P, inp["probes"])
    for f in (1, 2, 3):
        api("UpdateMaterial", P, np.int32(f), inp["sig"])
    for f in (4, 5, 6):
        api("UpdateMaterial", P, np.int32(f), inp["eps"])
    api("ReadySimulation", P)
    if mode == 5:
        api("SetIncidence", P, np.float64(ANG))
    api("Init1D", P, np.float32(1.0), inp["pw"])
    return P


def _oracle(inp, mode):
    import oracle

    o = oracle.OracleSim("f32")
    o.set_params(pml=PML, tfsf_width=W)
    o.set_const(inp["fr"], inp["td"])
    o.set_antenna_locations(inp["probes"])
    for f in (1, 2, 3):
        o.update_material(f, inp["sig"])
    for f in (4, 5, 6):
        o.update_material(f, inp["eps"])
    o.ready_simulation()
    if mode == 5:
        o.set_incidence(*ANG)
    o.init_1d(1.0, inp["pw"])
    for n in range(inp["steps"]):
        o.step(n, mode)
    return o


def _check(P, o, inp):
    from maxwell_solver_gb300 import simFDTD

    n = int(np.prod(DIMS))
    for f, name in zip(range(1, 7), FIELDS):
        got = simFDTD("OutputVis", P, np.uint32(n), np.int32(f))
        np.testing.assert_array_equal(got, o.field(name), err_msg=name)
    rec = simFDTD("OutputProbes", P, np.uint32(inp["steps"] * 6 * 6))
    np.testing.assert_array_equal(rec, o.array("probes"))
    assert np.abs(o.field("Ez")).max() > 0


@pytest.mark.parametrize("mode", [1, 2, 3, 4, 5])
def test_fused_step_equals_oracle(mode):
    """70 steps through StepN: two 32-step graph replays of fused pairs,
    then three single pairs."""
    from maxwell_solver_gb300 import info, simFDTD

    inp = _inputs(70)
    P = _ready(simFDTD, inp, mode)
    assert info(P)["fused"] == 1
    simFDTD("StepN", P, np.int32([0, inp["steps"], mode]))
    _check(P, _oracle(inp, mode), inp)
    simFDTD("DeleteSimulation", P)


def test_fused_per_op_calls_odd_count():
    """33 steps as the per-op calls of highfrequency.m: a held run of 32
    complete steps goes out as fused pairs, the last one the plain way."""
    from maxwell_solver_gb300 import simFDTD

    inp = _inputs(33)
    mode = 3
    P = _ready(simFDTD, inp, mode)
    for n in range(inp["steps"]):
        tm = np.array([n, mode], dtype=np.int32)
        simFDTD("UpdateH_All", P)
        simFDTD("UpdateH_PlaneWave", P, tm)
        simFDTD("UpdateH_PML", P)
        simFDTD("UpdateE_All", P)
        simFDTD("UpdateE_PlaneWave", P, tm)
        simFDTD("UpdateE_PML", P)
    _check(P, _oracle(inp, mode), inp)
    simFDTD("DeleteSimulation", P)


def test_fused_with_coefficient_arrays(monkeypatch):
    """Per-cell coefficient arrays (the reference's layout) instead of
    material ids: the pass reads them from global memory."""
    from maxwell_solver_gb300 import info, simFDTD

    monkeypatch.setenv("FDTD_COEF", "arrays")
    inp = _inputs(40)
    P = _ready(simFDTD, inp, 1)
    inf = info(P)
    assert inf["coef_mode"] == 0 and inf["fused"] == 1
    simFDTD("StepN", P, np.int32([0, inp["steps"], 1]))
    _check(P, _oracle(inp, 1), inp)
    simFDTD("DeleteSimulation", P)
