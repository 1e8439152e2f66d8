"""TF/SF mode 5 (oblique plane wave) on the GPU: bit-identical to the FP32
oracle's restatement (fields and probe record, spheres and CPML included),
within the stated tolerance of the FP64 build, the same through fdtd_step_n,
the per-op MEX calls and a batch, and with no leakage beyond the method's."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS, PML, W, STEPS = (46, 40, 44), 8, 12, 120
ANG = (math.radians(40), math.radians(25), math.radians(30))
FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _inputs(seed=21):
    from maxwell_solver_gb300.workloads import SHAPE_SPHERE, rasterize

    I, J, K = DIMS
    dx = 1e-3
    dt = 0.99 * dx / (math.sqrt(3) * 299792458.0)
    rows = [[SHAPE_SPHERE, 4.0, 0.02, 24.5, 19.0, 23.0, 5.5, 0, 0],
            [SHAPE_SPHERE, 2.5, 0.0, 16.0, 24.0, 28.0, 3.0, 0, 0]]
    eps, sig = rasterize(DIMS, 1.0, 0.0, rows)
    t = np.arange(STEPS) * np.float32(dt)
    f0, spread = 15e9, 20e-12
    pw = (np.sin(2 * np.pi * f0 * (t - 3 * spread)) *
          np.exp(-((t - 3 * spread) / spread) ** 2)).astype(np.float32)
    rng = np.random.default_rng(seed)
    probes = np.stack([rng.integers(1, d - 2 * PML - 1, 5) for d in DIMS], axis=1).astype(np.int32)
    return dict(fr=np.float32([f0, dx, dt]), td=np.int32([STEPS, I, J, K, 5]), eps=eps, sig=sig,
                pw=pw, probes=np.asfortranarray(probes))


def _ready(api, inp):
    P = api("CreateSimulation")
    api("SetParams", P, np.float64([PML, W, 3, 1, 0.08, 1, 0.8, 0]))
    api("SetConst", P, inp["fr"], inp["td"])
    api("SetAntennaLocations", P, inp["probes"])
    for f in (1, 2, 3):
        api("UpdateMaterial", P, np.int32(f), inp["sig"])
    for f in (4, 5, 6):
        api("UpdateMaterial", P, np.int32(f), inp["eps"])
    api("ReadySimulation", P)
    api("SetIncidence", P, np.float64(ANG))
    api("Init1D", P, np.float32(1.0), inp["pw"])
    return P


def _fields(api, P):
    n = int(np.prod(DIMS))
    return [api("OutputVis", P, np.uint32(n), np.int32(f)) for f in range(1, 7)]


def _oracle(inp, prec):
    import oracle

    o = oracle.OracleSim(prec)
    o.set_params(pml=PML, tfsf_width=W)
    o.set_const(inp["fr"], inp["td"])
    o.set_antenna_locations(inp["probes"])
    for f in (1, 2, 3):
        o.update_material(f, inp["sig"])
    for f in (4, 5, 6):
        o.update_material(f, inp["eps"])
    o.ready_simulation()
    o.set_incidence(*ANG)
    o.init_1d(1.0, inp["pw"])
    o.update_cuda()
    o.reset_field_all()
    for n in range(STEPS):
        o.step(n, 5)
    return o


def test_oblique_equals_oracle():
    from maxwell_solver_gb300 import simFDTD

    inp = _inputs()
    P = _ready(simFDTD, inp)
    simFDTD("StepN", P, np.int32([0, STEPS, 5]))
    got = _fields(simFDTD, P)
    probes = simFDTD("OutputProbes", P, np.uint32(STEPS * 5 * 6))
    o32, o64 = _oracle(inp, "f32"), _oracle(inp, "f64")
    for a, name in zip(got, FIELDS):
        np.testing.assert_array_equal(a, o32.field(name), err_msg=name)
    np.testing.assert_array_equal(probes, o32.array("probes"))
    for fam in (FIELDS[:3], FIELDS[3:]):
        ref = np.concatenate([o64.field(n) for n in fam])
        mine = np.concatenate([got[FIELDS.index(n)].astype(np.float64) for n in fam])
        assert np.linalg.norm(mine - ref) / np.linalg.norm(ref) <= 1e-5
    assert np.abs(got[2]).max() > 0.05
    simFDTD("DeleteSimulation", P)


def test_oblique_per_op_and_batch_equal_step_n(mex):
    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.batch import Batch

    inp = _inputs(seed=22)
    P = _ready(simFDTD, inp)
    simFDTD("StepN", P, np.int32([0, STEPS, 5]))
    want = _fields(simFDTD, P)
    Q = _ready(mex, inp)  # the reference's per-op call sequence through the MEX
    for n in range(STEPS):
        tm = np.int32([n, 5])
        mex("UpdateH_All", Q)
        mex("UpdateH_PlaneWave", Q, tm)
        mex("UpdateH_PML", Q)
        mex("UpdateE_All", Q)
        mex("UpdateE_PlaneWave", Q, tm)
        mex("UpdateE_PML", Q)
    for a, b in zip(_fields(mex, Q), want):
        np.testing.assert_array_equal(a, b)
    R = _ready(simFDTD, inp)
    S = _ready(simFDTD, _inputs(seed=23))
    with Batch() as b:
        b.add(R, 0, STEPS, 5)
        b.add(S, 0, STEPS // 2, 5)
        b.run()
    for a, c in zip(_fields(simFDTD, R), want):
        np.testing.assert_array_equal(a, c)
    for h in (P, R, S):
        simFDTD("DeleteSimulation", h)
    mex("DeleteSimulation", Q)


def test_oblique_without_incidence_is_refused():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    inp = _inputs()
    P = simFDTD("CreateSimulation")
    simFDTD("SetParams", P, np.float64([PML, W, 3, 1, 0.08, 1, 0.8, 0]))
    simFDTD("SetConst", P, inp["fr"], inp["td"])
    simFDTD("ReadySimulation", P)
    simFDTD("Init1D", P, np.float32(1.0), inp["pw"])
    with pytest.raises(SimFDTDError) as e:
        simFDTD("StepN", P, np.int32([0, 10, 5]))
    assert e.value.identifier == "simFDTD:InvalidState"
    simFDTD("DeleteSimulation", P)
