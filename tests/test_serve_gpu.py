"""Media as shapes and the serving loop.

SetShapes must give the same cells as the UpdateMaterial arrays built from
the same shapes (so every field bit matches), and a served request must end
with the same probes and fields whether it ran alone (a one-at-a-time queue)
or packed with others arriving at different times under a memory budget."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = range(1, 7)


def _small_specs(n, seed=11):
    from maxwell_solver_gb300.workloads import GridSpec, rng

    r = rng(seed)
    out = []
    for g in range(n):
        dims = tuple(int(x) for x in r.integers(36, 73, 3))
        steps, pml, mode = int(r.integers(60, 161)), int(r.integers(8, 11)), int(r.integers(1, 5))
        if g % 3 == 1:
            mode = 5  # oblique incidence, seeded angles
        out.append(GridSpec(dims, steps, pml, mode, int(r.integers(0, 6)),
                            float(r.uniform(10e9, 60e9)), seed * 1000 + g,
                            media="layers" if g % 3 == 2 else "spheres"))
    return out


def _ready(spec, shapes: bool):
    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.workloads import grid_materials, grid_shapes, grid_source

    I, J, K = spec.dims
    P = simFDTD("CreateSimulation")
    simFDTD("SetParams", P, np.float64([spec.pml, spec.pml + 5, 3, 1, 0.08, 1, 0.8, 0]))
    simFDTD("SetConst", P, np.float32([spec.fctr, spec.delX, spec.delT]),
            np.int32([spec.steps, I, J, K, 0]))
    if shapes:
        bg_e, bg_s, rows = grid_shapes(spec)
        simFDTD("SetShapes", P, np.float32([bg_e, bg_s]), np.array(rows, dtype=np.float64))
    else:
        eps, sig = grid_materials(spec)
        for f in (1, 2, 3):
            simFDTD("UpdateMaterial", P, np.int32(f), sig)
        for f in (4, 5, 6):
            simFDTD("UpdateMaterial", P, np.int32(f), eps)
    simFDTD("ReadySimulation", P)
    if spec.mode == 5:
        simFDTD("SetIncidence", P, np.float64(spec.angles))
    simFDTD("Init1D", P, np.float32(1.0), grid_source(spec))
    return P


@pytest.mark.parametrize("media", ["spheres", "layers"])
def test_shapes_equal_material_arrays(media):
    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.workloads import GridSpec, grid_materials

    spec = GridSpec((57, 49, 66), 90, 9, 3, 6, 30e9, 4242, media=media)
    n = int(np.prod(spec.dims))
    out = []
    for shapes in (True, False):
        P = _ready(spec, shapes)
        simFDTD("StepN", P, np.int32([0, spec.steps, spec.mode]))
        out.append([simFDTD("OutputVis", P, np.uint32(n), np.int32(f)) for f in FIELDS])
        if shapes:  # OutputVis of the media follows the shapes
            eps, sig = grid_materials(spec)
            np.testing.assert_array_equal(simFDTD("OutputVis", P, np.uint32(n), np.int32(-4)), eps)
            np.testing.assert_array_equal(simFDTD("OutputVis", P, np.uint32(n), np.int32(0)), sig)
        simFDTD("DeleteSimulation", P)
    assert np.abs(out[1][2]).max() > 0
    for a, b, f in zip(out[0], out[1], FIELDS):
        np.testing.assert_array_equal(a, b, err_msg=f"field {f}")


def _serve(specs, gaps, **cfg):
    from maxwell_solver_gb300.serve import Server

    with Server(**cfg) as srv:
        tickets = []
        for spec, gap in zip(specs, gaps):
            time.sleep(gap)
            tickets.append(srv.submit(spec, n_probes=6, out_field=3))
        res = [srv.result(t) for t in tickets]
        st = srv.stats()
    return res, st


@pytest.mark.parametrize("policy", ["srpt", "hrrn", "bounded", "deadline"])
def test_served_results_equal_alone(policy):
    """Requests arriving while others run are packed into the same batched
    launches (in either order policy); each ends bit-identical to running
    alone."""
    from maxwell_solver_gb300.serve import estimate_device_bytes

    specs = _small_specs(9)
    est = [estimate_device_bytes(s, 6) for s in specs]
    budget = int(max(est) + 0.6 * (sum(est) - max(est)))  # some requests must queue
    rng = np.random.default_rng(5)
    gaps = rng.exponential(0.01, len(specs))  # Poisson arrivals
    mixed, st = _serve(specs, gaps, hbm_budget=budget, round_steps=16, policy=policy)
    alone, st1 = _serve(specs, [0.0] * len(specs), hbm_budget=budget, one_at_a_time=True)
    assert st["completed"] == len(specs) and st["failed"] == 0
    assert st["peak_reserved_bytes"] <= budget
    assert st["peak_active"] >= 2  # solves overlapped on the device
    assert st1["peak_active"] == 1
    assert st["latency_p50_s"] <= st["latency_p90_s"] <= st["latency_p99_s"]
    for spec, a, b in zip(specs, mixed, alone):
        assert np.abs(a["field"]).max() > 0, spec
        np.testing.assert_array_equal(a["field"], b["field"], err_msg=str(spec))
        np.testing.assert_array_equal(a["probes"], b["probes"], err_msg=str(spec))


def test_solo_rounds_equal_alone():
    """With a solo threshold inside the mix the larger requests run alone
    through fdtd_step_n between batched rounds of the smaller ones; every
    result still equals the one-at-a-time run."""
    specs = _small_specs(8, seed=17)
    cells = sorted(int(np.prod(s.dims)) for s in specs)
    solo = cells[len(cells) // 2]
    mixed, st = _serve(specs, [0.0] * len(specs), hbm_budget=16 << 30, round_steps=16,
                       solo_cells=solo)
    alone, _ = _serve(specs, [0.0] * len(specs), hbm_budget=16 << 30, one_at_a_time=True)
    assert st["completed"] == len(specs) and st["failed"] == 0
    for spec, a, b in zip(specs, mixed, alone):
        np.testing.assert_array_equal(a["field"], b["field"], err_msg=str(spec))
        np.testing.assert_array_equal(a["probes"], b["probes"], err_msg=str(spec))


def test_served_result_equals_plain_handle():
    """One request through the server equals the same solve set up by hand
    (shapes) and run with StepN."""
    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.workloads import grid_probes

    spec = _small_specs(1, seed=23)[0]
    (res,), _ = _serve([spec], [0.0], hbm_budget=8 << 30)
    P = _ready_with_probes(spec, grid_probes(spec, 6))
    simFDTD("StepN", P, np.int32([0, spec.steps, spec.mode]))
    n = int(np.prod(spec.dims))
    np.testing.assert_array_equal(res["field"], simFDTD("OutputVis", P, np.uint32(n), np.int32(3)))
    np.testing.assert_array_equal(res["probes"],
                                  simFDTD("OutputProbes", P, np.uint32(spec.steps * 6 * 6)))
    simFDTD("DeleteSimulation", P)


def _ready_with_probes(spec, probes):
    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.workloads import grid_shapes, grid_source

    I, J, K = spec.dims
    P = simFDTD("CreateSimulation")
    simFDTD("SetParams", P, np.float64([spec.pml, spec.pml + 5, 3, 1, 0.08, 1, 0.8, 0]))
    simFDTD("SetConst", P, np.float32([spec.fctr, spec.delX, spec.delT]),
            np.int32([spec.steps, I, J, K, probes.shape[0]]))
    bg_e, bg_s, rows = grid_shapes(spec)
    simFDTD("SetShapes", P, np.float32([bg_e, bg_s]), np.array(rows, dtype=np.float64))
    simFDTD("SetAntennaLocations", P, np.asfortranarray(probes).ravel(order="F"))
    simFDTD("ReadySimulation", P)
    if spec.mode == 5:
        simFDTD("SetIncidence", P, np.float64(spec.angles))
    simFDTD("Init1D", P, np.float32(1.0), grid_source(spec))
    return P


def test_request_over_budget_fails_alone():
    from maxwell_solver_gb300 import SimFDTDError
    from maxwell_solver_gb300.serve import Server, estimate_device_bytes

    small, big = _small_specs(2, seed=31)
    budget = estimate_device_bytes(small, 6) + 1
    if estimate_device_bytes(big, 6) <= budget:
        big = type(big)((72, 72, 72), big.steps, big.pml, big.mode, 0, big.fctr, big.seed)
    with Server(hbm_budget=budget) as srv:
        tb = srv.submit(big, n_probes=6)
        ts = srv.submit(small, n_probes=6)
        with pytest.raises(SimFDTDError) as e:
            srv.result(tb)
        assert "FDTD_ERR_OOM" in str(e.value)
        assert srv.result(ts)["info"]["status"] == 0
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1


def test_budget_from_free_device_memory():
    """hbm_budget 0: the server admits by the device memory free when it was
    created (90 % of it)."""
    import torch

    from maxwell_solver_gb300.serve import Server

    spec = _small_specs(1, seed=41)[0]
    with Server(hbm_budget=0) as srv:
        t = srv.submit(spec, n_probes=6)
        res = srv.result(t)
        st = srv.stats()
    free, total = torch.cuda.mem_get_info()
    assert 0 < st["hbm_budget"] <= total
    assert st["hbm_budget"] >= 0.5 * free  # most of what is free now
    assert res["info"]["status"] == 0 and st["completed"] == 1
