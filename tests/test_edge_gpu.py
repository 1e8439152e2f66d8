"""Edge cases and error behaviour of the drop-in interface on the GPU:
the reference's error identifiers, its soft-misuse paths, calls out of the
usual order, readout sizes, and the boundary quirks the reference has (last
x-plane coefficients, never-updated H faces)."""
import numpy as np
import pytest

from scenarios import by_name, run_mex, run_oracle

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def small_sim(api, dims=(32, 34, 36), T=20, n_ant=0, mode=True):
    sc = by_name("hf_mode3_vacuum")
    I, J, K = dims
    P = api("CreateSimulation")
    api("SetConst", P, np.float32([30e9, 1e-3, sc.delT]), np.int32([T, I, J, K, n_ant]))
    api("SetSource", P, np.ones(T, dtype=np.float32))
    if n_ant:
        api("SetAntennaLocations", P, np.int32([[1, 2, 3]] * n_ant))
    api("ReadySimulation", P)
    if mode:
        api("Init1D", P, np.float32(1), np.sin(np.arange(T, dtype=np.float32) * 0.3))
    return P


def test_reference_error_identifiers():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    P = small_sim(simFDTD)
    with pytest.raises(SimFDTDError) as e:
        simFDTD("SetConst", P, np.float32([1, 1e-3, 1e-12]), np.int32([5, 32, 32, 32, 0]))
    assert e.value.identifier == "simFDTD:AlreadyInitialized"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("Frobnicate", P)
    assert e.value.identifier == "simFDTD:UnknownOperation"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("AddCurrents", P, np.int32([0, 1]))
    assert e.value.identifier == "simFDTD:InvalidInput"
    simFDTD("DeleteSimulation", P)
    with pytest.raises(SimFDTDError) as e:  # use after delete
        simFDTD("UpdateH_All", P)
    assert e.value.identifier == "simFDTD:InvalidHandle"


def test_out_of_order_and_out_of_range():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    P = simFDTD("CreateSimulation")
    with pytest.raises(SimFDTDError) as e:
        simFDTD("UpdateH_All", P)  # before SetConst / ReadySimulation
    assert e.value.identifier == "simFDTD:InvalidState"
    simFDTD("SetConst", P, np.float32([30e9, 1e-3, 1.9e-12]), np.int32([10, 32, 32, 32, 0]))
    with pytest.raises(SimFDTDError) as e:
        simFDTD("Init1D", P, np.float32(1), np.ones(10, np.float32))  # before ReadySimulation
    assert e.value.identifier == "simFDTD:InvalidState"
    simFDTD("ReadySimulation", P)
    with pytest.raises(SimFDTDError) as e:
        simFDTD("UpdateH_PlaneWave", P, np.int32([0, 3]))  # before Init1D
    assert e.value.identifier == "simFDTD:InvalidState"
    simFDTD("Init1D", P, np.float32(1), np.ones(10, np.float32))
    with pytest.raises(SimFDTDError) as e:
        simFDTD("UpdateE_PlaneWave", P, np.int32([10, 3]))  # step == T
    assert e.value.identifier == "simFDTD:InvalidInput"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("AddCurrents", P, np.int32([0, 1]), np.int32([1, 2, 1, 2, 1, 2]))  # no source
    assert e.value.identifier == "simFDTD:InvalidState"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("SetAntennaLocations", P, np.int32([1, 1, 1]))  # after ReadySimulation
    assert e.value.identifier == "simFDTD:InvalidState"
    with pytest.raises(SimFDTDError) as e:
        simFDTD("UpdateMaterial", P, np.int32(1), np.zeros(5, np.float32))  # too short
    assert e.value.identifier == "simFDTD:InvalidInput"
    simFDTD("DeleteSimulation", P)


def test_grid_too_small_is_rejected():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    P = simFDTD("CreateSimulation")
    with pytest.raises(SimFDTDError) as e:
        simFDTD("SetConst", P, np.float32([1, 1e-3, 1e-12]), np.int32([5, 20, 40, 40, 0]))
    assert e.value.identifier == "simFDTD:Unsupported"
    simFDTD("DeleteSimulation", P)


def test_soft_misuse_matches_reference():
    """Reference behaviours that print and continue: a second SetSource is
    ignored, unknown UpdateMaterial flags / plane-wave modes / current modes do
    nothing, a current box with a negative or reversed range touches nothing,
    OutputAnt without antennas returns zeros."""
    from maxwell_solver_gb300 import simFDTD

    P = small_sim(simFDTD)
    ijk = 32 * 34 * 36
    simFDTD("SetSource", P, np.full(20, 5.0, np.float32))  # ignored
    simFDTD("UpdateMaterial", P, np.int32(9), np.zeros(ijk, np.float32))
    simFDTD("UpdateH_PlaneWave", P, np.int32([0, 7]))
    simFDTD("AddCurrents", P, np.int32([0, 5]), np.int32([1, 2, 1, 2, 1, 2]))
    simFDTD("AddCurrents", P, np.int32([0, 1]), np.int32([-1, 5, 1, 2, 1, 2]))
    simFDTD("AddCurrents", P, np.int32([0, 1]), np.int32([5, 1, 1, 2, 1, 2]))
    for f in range(1, 7):
        assert not simFDTD("OutputVis", P, np.uint32(ijk), np.int32(f)).any()
    simFDTD("AddCurrents", P, np.int32([0, 1]), np.int32([4, 6, 5, 5, 7, 7]))
    ex = simFDTD("OutputVis", P, np.uint32(ijk), np.int32(1))
    # source 1 (the first SetSource): E -= Cexh * 1 * dx / dx / dx on 3 cells
    assert np.count_nonzero(ex) == 3
    assert not simFDTD("OutputAnt", P, np.uint32(10)).any()
    simFDTD("DeleteSimulation", P)


def test_output_vis_sizes_and_flags():
    from maxwell_solver_gb300 import simFDTD

    P = small_sim(simFDTD)
    ijk = 32 * 34 * 36
    sig = np.linspace(0, 1, ijk).astype(np.float32)
    simFDTD("UpdateMaterial", P, np.int32(2), sig)
    np.testing.assert_array_equal(simFDTD("OutputVis", P, np.uint32(ijk), np.int32(-1)), sig)
    short = simFDTD("OutputVis", P, np.uint32(100), np.int32(-1))
    np.testing.assert_array_equal(short, sig[:100])
    long = simFDTD("OutputVis", P, np.uint32(ijk + 50), np.int32(-1))
    np.testing.assert_array_equal(long[:ijk], sig)
    assert not long[ijk:].any()
    eps = np.full(ijk, 2.5, np.float32)
    simFDTD("UpdateMaterial", P, np.int32(6), eps)
    np.testing.assert_array_equal(simFDTD("OutputVis", P, np.uint32(ijk), np.int32(-5)), eps)
    assert not simFDTD("OutputVis", P, np.uint32(ijk), np.int32(42)).any()
    simFDTD("DeleteSimulation", P)


def test_boundary_quirks_match_oracle():
    """The last x-plane has Cexh=Ceyh=Cezh=0 (den_ex stops at Imax-2) and the
    H max faces are never updated; E there still evolves as the reference."""
    from maxwell_solver_gb300 import simFDTD

    sc = by_name("gic_currents_x")
    inp = sc.inputs()
    P = run_mex(simFDTD, sc, inp)
    I, J, K = sc.dims
    ijk = I * J * K
    o = run_oracle(sc, "f32", inp=inp)
    for f, n in zip(range(1, 7), FIELDS):
        got = simFDTD("OutputVis", P, np.uint32(ijk), np.int32(f)).reshape((I, J, K), order="F")
        want = o.field(n).reshape((I, J, K), order="F")
        np.testing.assert_array_equal(got, want)
        if n.startswith("H"):
            assert not got[I - 1].any() and not got[:, J - 1].any() and not got[:, :, K - 1].any()
    simFDTD("DeleteSimulation", P)


def test_reset_replays_identically():
    from maxwell_solver_gb300 import simFDTD

    sc = by_name("mode1_spheres")
    inp = sc.inputs()
    P = run_mex(simFDTD, sc, inp)
    ijk = int(np.prod(sc.dims))
    first = [simFDTD("OutputVis", P, np.uint32(ijk), np.int32(f)) for f in range(1, 7)]
    simFDTD("ResetFieldAll", P)
    simFDTD("StepN", P, np.int32([0, sc.steps, sc.mode]))
    second = [simFDTD("OutputVis", P, np.uint32(ijk), np.int32(f)) for f in range(1, 7)]
    for a, b in zip(first, second):
        np.testing.assert_array_equal(a, b)
    simFDTD("DeleteSimulation", P)


def test_update_cuda_takes_new_materials():
    """UpdateMaterial only takes effect at UpdateCuda (src/simulation.h:288-328,
    :1097-1127): same result as the oracle following the same sequence."""
    from maxwell_solver_gb300 import simFDTD
    from oracle import OracleSim

    sc = by_name("hf_mode3_vacuum")
    inp = sc.inputs()
    P = run_mex(simFDTD, type(sc)(**{**sc.__dict__, "steps": 0}), inp)
    o = OracleSim("f32")
    o.set_const(inp["freqRes"], inp["TimeDim"])
    o.set_source(inp["source"])
    o.ready_simulation()
    o.init_1d(1.0, inp["pw"])
    ijk = int(np.prod(sc.dims))
    sig = np.full(ijk, 0.05, np.float32)
    for api_step in range(2):
        simFDTD("UpdateMaterial", P, np.int32(3), sig)
        o.update_material(3, sig)
        if api_step == 1:
            simFDTD("UpdateCuda", P)
            o.update_cuda()
        for n in range(20 * api_step, 20 * api_step + 20):
            simFDTD("StepN", P, np.int32([n, 1, 3]))
            o.step(n, 3)
    for f, n in zip(range(1, 7), FIELDS):
        np.testing.assert_array_equal(simFDTD("OutputVis", P, np.uint32(ijk), np.int32(f)),
                                      o.field(n))
    simFDTD("DeleteSimulation", P)


def test_create_mu_after_ready_leaves_h_update_unchanged():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    P = simFDTD("CreateSimulation")
    simFDTD("SetConst", P, np.float32([30e9, 1e-3, 1.9e-12]), np.int32([4, 32, 32, 32, 0]))
    ijk = 32 ** 3
    with pytest.raises(SimFDTDError) as e:
        simFDTD("CreateMu", P, *(np.ones(ijk, np.float32),) * 3)
    assert e.value.identifier == "simFDTD:InvalidState"
    simFDTD("DeleteSimulation", P)
    sc = by_name("curl_only_currents_z")
    inp = sc.inputs()
    ref = run_mex(simFDTD, sc, inp)
    n = int(np.prod(sc.dims))
    want = [simFDTD("OutputVis", ref, np.uint32(n), np.int32(f)) for f in range(1, 7)]
    sc0 = type(sc)(**{**sc.__dict__, "steps": 0})
    P = run_mex(simFDTD, sc0, inp)
    simFDTD("CreateMu", P, *(np.full(n, 2.0, np.float32),) * 3)
    for s in range(sc.steps):
        simFDTD("UpdateH_All", P)
        simFDTD("UpdateE_All", P)
        simFDTD("AddCurrents", P, np.int32([s, sc.cur_mode]), np.int32(sc.cur_box))
    got = [simFDTD("OutputVis", P, np.uint32(n), np.int32(f)) for f in range(1, 7)]
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    simFDTD("DeleteSimulation", P)
    simFDTD("DeleteSimulation", ref)


def test_probe_rows_follow_update_h_all():
    """Row r of the probe record = fields at the start of step r; rows after
    the last step stay zero; ResetFieldAll rewinds the recorder."""
    from maxwell_solver_gb300 import simFDTD

    P = small_sim(simFDTD, T=12, n_ant=2)
    for n in range(5):
        simFDTD("UpdateH_All", P)
        simFDTD("UpdateH_PlaneWave", P, np.int32([n, 3]))
        simFDTD("UpdateE_All", P)
        simFDTD("UpdateE_PlaneWave", P, np.int32([n, 3]))
    rec = simFDTD("OutputProbes", P, np.uint32(12 * 2 * 6)).reshape(12, 2, 6)
    assert not rec[0].any()          # start of step 0: zero fields
    assert not rec[5:].any()         # never recorded
    simFDTD("ResetFieldAll", P)
    simFDTD("UpdateH_All", P)
    rec2 = simFDTD("OutputProbes", P, np.uint32(12 * 2 * 6)).reshape(12, 2, 6)
    assert not rec2[0].any()
    np.testing.assert_array_equal(rec2[1:5], rec[1:5])
    simFDTD("DeleteSimulation", P)
