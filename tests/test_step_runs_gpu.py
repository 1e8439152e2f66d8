"""The per-op calls in the reference's step order are held and reach the
device as whole steps (graph replays, like fdtd_step_n).  Readouts in the
middle of a run, a current source on some steps, steps without TF/SF, a
mode switch, a step whose PlaneWave call is missing and run lengths that
are not a multiple of the graph's step count must all give exactly what
issuing every step on its own gives (fdtd_step_n one step at a time)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS, T = (40, 36, 38), 100
BOX = np.int32([19, 20, 17, 18, 16, 20])


def _sim(api):
    from scenarios import by_name

    sc = by_name("hf_mode3_vacuum")
    I, J, K = DIMS
    P = api("CreateSimulation")
    api("SetConst", P, np.float32([30e9, 1e-3, sc.delT]), np.int32([T, I, J, K, 4]))
    t = np.arange(T, dtype=np.float32)
    api("SetSource", P, np.exp(-((t - 50) / 12) ** 2).astype(np.float32))
    api("SetAntennaLocations", P, np.int32([[1, 2, 3], [5, 6, 7], [9, 4, 2], [10, 10, 10]]))
    api("ReadySimulation", P)
    api("Init1D", P, np.float32(1), np.sin(t * 0.3).astype(np.float32))
    return P


def _plan(n):
    """(tfsf mode, current?, PlaneWave calls made?) of step n."""
    if 45 <= n < 60:
        return 3, True, True
    if 60 <= n < 70:
        return 0, False, False
    if 80 <= n < 90:
        return 1, False, True
    return 3, False, True  # (step 92: the E PlaneWave call is left out below)


def _fields(api, P):
    n = int(np.prod(DIMS))
    return [api("OutputVis", P, np.uint32(n), np.int32(f)) for f in range(1, 7)]


def test_held_runs_equal_single_steps():
    from maxwell_solver_gb300 import simFDTD

    P = _sim(simFDTD)
    mid = None
    for n in range(T):
        mode, cur, pw = _plan(n)
        tm = np.int32([n, mode])
        simFDTD("UpdateH_All", P)
        if pw and mode:
            simFDTD("UpdateH_PlaneWave", P, tm)
        simFDTD("UpdateH_PML", P)
        simFDTD("UpdateE_All", P)
        if pw and mode and n != 92:
            simFDTD("UpdateE_PlaneWave", P, tm)
        simFDTD("UpdateE_PML", P)
        if cur:
            simFDTD("AddCurrents", P, np.int32([n, 2]), BOX)
        if n == 40:  # steps 0-31 went as one graph replay; a readout mid-run
            mid = _fields(simFDTD, P)
    got = _fields(simFDTD, P)
    rec = simFDTD("OutputProbes", P, np.uint32(T * 4 * 6))
    simFDTD("DeleteSimulation", P)

    Q = _sim(simFDTD)
    for n in range(T):
        mode, cur, pw = _plan(n)
        if n == 92:  # H with TF/SF, E without: two explicit half-steps
            simFDTD("UpdateH_All", Q)
            simFDTD("UpdateH_PlaneWave", Q, np.int32([n, mode]))
            simFDTD("UpdateH_PML", Q)
            simFDTD("Synchronize", Q)
            simFDTD("UpdateE_All", Q)
            simFDTD("UpdateE_PML", Q)
            simFDTD("Synchronize", Q)
            continue
        args = [np.int32([n, 1, mode if pw else 0])]
        if cur:
            args.append(np.int32([2, *BOX]))
        simFDTD("StepN", Q, *args)
        if n == 40:
            for a, b in zip(_fields(simFDTD, Q), mid):
                np.testing.assert_array_equal(a, b)
    want = _fields(simFDTD, Q)
    ref = simFDTD("OutputProbes", Q, np.uint32(T * 4 * 6))
    simFDTD("DeleteSimulation", Q)
    assert np.abs(got[2]).max() > 0
    for a, b, name in zip(got, want, ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
        np.testing.assert_array_equal(a, b, err_msg=name)
    np.testing.assert_array_equal(rec, ref)
