"""The library against the reference's own CUDA kernels on the same GPU.

tests/refgpu.py runs the reference's kernels (src/gpu.h, compiled for
sm_103a by oracle/ref_gpu_build.py) with the reference's launch shapes over
the CPU oracle's set-up.  Built without multiply-add contraction they
evaluate every expression the way the library does, so the fields must be
equal bit for bit.  Built with the reference's own flags (contraction on,
src/Compile.m:4-6) they round differently in the last bit of many
operations, so the two runs drift apart by rounding noise: the E and H
fields, each taken as one vector of its three components, agree to a
relative L2 error of at most 1e-5.  (Per component the figure means
little where a component is itself rounding noise, as the TF/SF leakage
into Ex of a mode-3 run is.)  The last test times both on the
512 x 512 x 448 workload.
"""
import json
import os
import time

import numpy as np
import pytest

from refgpu import unavailable
from scenarios import SCENARIOS, run_mex

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
REL_L2 = 1e-5  # E and H against the contracted build; the uncontracted one is exact


@pytest.fixture(scope="module", autouse=True)
def _need_reference_kernels():
    why = unavailable()
    if why:
        pytest.skip(f"reference kernels: {why}")


def _ours(P, n):
    from maxwell_solver_gb300 import simFDTD

    return {f: simFDTD("OutputVis", P, np.uint32(n), np.int32(i + 1))
            for i, f in enumerate(FIELDS)}


def _rel_l2(a, b):
    d = np.linalg.norm(a.astype(np.float64) - b.astype(np.float64))
    n = np.linalg.norm(b.astype(np.float64))
    return d / n if n > 0 else d


def _family_errors(ours, ref):
    """Relative L2 error of E = (Ex, Ey, Ez) and of H = (Hx, Hy, Hz)."""
    out = {}
    for fam in ("E", "H"):
        names = [fam + c for c in "xyz"]
        out[fam] = _rel_l2(np.concatenate([ours[n] for n in names]),
                           np.concatenate([ref[n] for n in names]))
    return out


@pytest.mark.parametrize("sc", SCENARIOS, ids=[s.name for s in SCENARIOS])
def test_scenarios_equal_reference_kernels(sc):
    """Every scenario (modes 1-4, current sources, probes): bit-identical to
    the reference's kernels without contraction, within REL_L2 with it."""
    from maxwell_solver_gb300 import simFDTD
    from refgpu import RefGPU

    inp = sc.inputs()
    P = run_mex(simFDTD, sc, inp)
    got = _ours(P, int(np.prod(sc.dims)))
    simFDTD("DeleteSimulation", P)
    for fma in (False, True):
        ref = RefGPU(fma=fma)
        run_mex(ref, sc, inp)
        r = {f: ref.field(f) for f in FIELDS}
        ref.close()
        if not fma:
            for f in FIELDS:
                np.testing.assert_array_equal(got[f], r[f], err_msg=f"{sc.name} {f}")
    err = _family_errors(got, r)
    print(json.dumps({"scenario": sc.name, "contracted_rel_l2": err}))
    assert max(err.values()) <= REL_L2, (sc.name, err)


def _run_workload(name, steps, timed=0):
    """The workload through the library and through the reference's kernels
    (contraction off, then on, from the same set-up); returns the fields of
    each after `steps` steps and, with timed > 0, the seconds per step of
    the last `timed` of them."""
    import torch

    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.workloads import WORKLOADS, setup
    from refgpu import RefGPU

    w = WORKLOADS[name]
    n = w.cells
    P = setup(simFDTD, w, steps=steps)
    warm = steps - timed
    simFDTD("StepN", P, np.int32([0, warm, w.mode]))
    simFDTD("Synchronize", P)
    t0 = time.perf_counter()
    if timed:
        simFDTD("StepN", P, np.int32([warm, timed, w.mode]))
        simFDTD("Synchronize", P)
    ours_s = (time.perf_counter() - t0) / max(timed, 1)
    ours = _ours(P, n)
    simFDTD("DeleteSimulation", P)

    ref = RefGPU(fma=False)
    setup(ref, w, steps=steps)
    out = {}
    ref_s = None
    for fma in (False, True):
        ref.load(fma)
        ref("ResetFieldAll")
        for k in range(warm):
            ref.step(k, w.mode)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for k in range(warm, steps):
            ref.step(k, w.mode)
        ev1.record()
        torch.cuda.synchronize()
        if fma and timed:
            ref_s = ev0.elapsed_time(ev1) * 1e-3 / timed
        out[fma] = {f: ref.field(f) for f in FIELDS}
    ref.close()
    return ours, out, ours_s, ref_s


def _ref_graph_s_per_step(name, steps, timed):
    """Device time per step of the reference's kernels with launch costs
    taken out: the last `timed` steps captured into one CUDA graph and
    replayed (the most favourable measure for the reference, whose own
    loop launches its twelve kernels per step one by one)."""
    import torch

    from maxwell_solver_gb300.workloads import WORKLOADS, setup
    from refgpu import RefGPU

    w = WORKLOADS[name]
    ref = RefGPU(fma=True)
    setup(ref, w, steps=steps)
    ref("ResetFieldAll")
    for k in range(steps - timed):
        ref.step(k, w.mode)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    ref.stream = side.cuda_stream
    with torch.cuda.graph(graph, stream=side):
        for k in range(steps - timed, steps):
            ref.step(k, w.mode)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    graph.replay()
    ev1.record()
    torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) * 1e-3 / timed
    del graph
    ref.close()
    return sec


def _report(rep):
    """Prints the comparison; with FDTD_REF_GPU_REPORT=path also merges it
    into that JSON file, keyed by workload."""
    print(json.dumps(rep))
    path = os.environ.get("FDTD_REF_GPU_REPORT")
    if path:
        allrep = {}
        if os.path.exists(path):
            with open(path) as fh:
                allrep = json.load(fh)
        allrep[rep["workload"].split()[0]] = rep
        with open(path, "w") as fh:
            json.dump(allrep, fh)


def test_c1_full_run_equals_reference_kernels():
    """64^3, 10-cell CPML, TF/SF mode 3, 500 steps (the last 400 timed)."""
    from maxwell_solver_gb300.workloads import WORKLOADS

    timed = 400
    ours, ref, ours_s, _ = _run_workload("c1", 500, timed)
    ref_s = _ref_graph_s_per_step("c1", 500, timed)
    for fam in ("E", "H"):
        assert max(np.abs(ours[fam + c]).max() for c in "xyz") > 0
    for f in FIELDS:
        np.testing.assert_array_equal(ours[f], ref[False][f], err_msg=f)
    err = _family_errors(ours, ref[True])
    cells = WORKLOADS["c1"].cells
    _report({"workload": "c1 64^3, 10-cell CPML, vacuum, TF/SF mode 3", "steps": 500,
             "steps_timed": timed,
             "reference_kernels_ms_per_step": round(ref_s * 1e3, 4),
             "reference_kernels_Mcell_steps_per_s": round(cells / ref_s / 1e6, 1),
             "library_ms_per_step": round(ours_s * 1e3, 4),
             "library_Mcell_steps_per_s": round(cells / ours_s / 1e6, 1),
             "speedup": round(ref_s / ours_s, 2), "contracted_rel_l2": err,
             "timing": "reference: its 400 steps (12 launches each) captured into one CUDA "
                       "graph and replayed, CUDA events around the replay (device time only); "
                       "library: wall clock around fdtd_step_n of 400 steps"})
    assert max(err.values()) <= REL_L2, err


def test_c3_equals_and_outruns_reference_kernels():
    """512 x 512 x 448, 16-cell CPML, six layers, TF/SF mode 1: 288 steps
    (the pulse enters the grid after about 130) equal to the reference's
    kernels, and the step time of both over the last 32 (inputs far larger
    than L2)."""
    from maxwell_solver_gb300.workloads import WORKLOADS

    timed = 32
    ours, ref, ours_s, ref_s = _run_workload("c3", 288, timed)
    for fam in ("E", "H"):  # the comparison is not of empty grids
        assert max(np.abs(ours[fam + c]).max() for c in "xyz") > 0
    for f in FIELDS:
        np.testing.assert_array_equal(ours[f], ref[False][f], err_msg=f)
    err = _family_errors(ours, ref[True])
    cells = WORKLOADS["c3"].cells
    rep = {"workload": "c3 512x512x448, 16-cell CPML, 6 layers, TF/SF mode 1",
           "steps": 288, "steps_timed": timed,
           "reference_kernels_ms_per_step": round(ref_s * 1e3, 4),
           "reference_kernels_Mcell_steps_per_s": round(cells / ref_s / 1e6, 1),
           "library_ms_per_step": round(ours_s * 1e3, 4),
           "library_Mcell_steps_per_s": round(cells / ours_s / 1e6, 1),
           "speedup": round(ref_s / ours_s, 2),
           "contracted_rel_l2": err,
           "timing": "reference: CUDA events around its 32 steps of kernel launches "
                     "(12 per step, the reference's launch shapes); library: wall clock "
                     "around fdtd_step_n of 32 steps and a synchronize (probe gather included)"}
    _report(rep)
    assert max(err.values()) <= REL_L2, err
    assert ours_s < ref_s


def test_probe_record_samples_reference_kernel_fields():
    """The probe record (row n: the six fields at each probe at the start of
    step n) holds exactly the reference kernels' fields at the probe cells,
    whose linear index is the reference's coax index: (pml + x) + (pml + y)
    Imax + (pml + z) Imax Jmax (src/simulation.h:1047-1067; the reference
    allocates the record but no kernel of it writes one)."""
    import torch

    from maxwell_solver_gb300 import simFDTD
    from refgpu import RefGPU
    from scenarios import by_name

    sc = by_name("mode3_probes_y_current")
    inp = sc.inputs()
    P = run_mex(simFDTD, sc, inp)
    rec = simFDTD("OutputProbes", P, np.uint32(sc.steps * sc.n_probes * 6))
    simFDTD("DeleteSimulation", P)
    rec = rec.reshape(sc.steps, sc.n_probes, 6)

    I, J, _ = sc.dims
    p = 10  # the scenarios keep the reference's CPML thickness
    loc = np.asarray(inp["probes"], dtype=np.int64)
    idx = torch.as_tensor((p + loc[:, 0]) + (p + loc[:, 1]) * I + (p + loc[:, 2]) * I * J,
                          device="cuda")
    ref = RefGPU(fma=False)
    rows = [np.zeros((sc.n_probes, 6), dtype=np.float32)]  # the state before step 0

    def sample(n, _P):
        if n + 1 < sc.steps:
            rows.append(torch.stack([ref.d[f][idx] for f in FIELDS], dim=1).cpu().numpy())

    run_mex(ref, sc, inp, on_step=sample)
    ref.close()
    np.testing.assert_array_equal(rec, np.stack(rows))
    assert np.abs(rec).max() > 0
