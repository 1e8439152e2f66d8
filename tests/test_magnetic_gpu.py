"""Per-cell magnetic media (fdtd_set_magnetic / 'SetMagnetic') on the GPU:
bit-identical to the FP32 oracle (fields and probe record) with mu_r and
sigma_m regions crossing a TF/SF face and a CPML slab, in an axis mode and
the oblique mode, with the coefficients indexed (few distinct values) and as
per-cell arrays (one value per cell); within the stated tolerance of the
FP64 build; the same through the per-op MEX calls; mu_r = 1, sigma_m = 0
reproduces the default update exactly."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS, PML, W, STEPS = (46, 40, 44), 8, 12, 100
ANG = (math.radians(55), math.radians(20), math.radians(70))
FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _inputs(per_cell=False, seed=31):
    from maxwell_solver_gb300.workloads import SHAPE_SPHERE, rasterize

    I, J, K = DIMS
    dx = 1e-3
    dt = 0.99 * dx / (math.sqrt(3) * 299792458.0)
    eps, sig = rasterize(DIMS, 1.0, 0.0, [[SHAPE_SPHERE, 3.0, 0.01, 26.0, 20.0, 22.0, 5.0, 0, 0]])
    # mu_r / sigma_m: a sphere across the low-x TF/SF face, one in the CPML
    # corner, one inside the box
    rows = [[SHAPE_SPHERE, 3.0, 0.0, 12.0, 20.0, 22.0, 5.0, 0, 0],
            [SHAPE_SPHERE, 2.0, 2.0e3, 5.0, 30.0, 30.0, 4.0, 0, 0],
            [SHAPE_SPHERE, 1.5, 5.0e2, 30.0, 22.0, 26.0, 4.5, 0, 0]]
    mu, sm = rasterize(DIMS, 1.0, 0.0, rows)
    rng = np.random.default_rng(seed)
    if per_cell:  # one distinct tuple per cell: the per-cell arrays
        mu = [(mu * rng.uniform(1.0, 1.5, mu.size)).astype(np.float32) for _ in range(3)]
        sm = [(sm + rng.uniform(0.0, 50.0, sm.size)).astype(np.float32) for _ in range(3)]
    else:
        mu, sm = [mu] * 3, [sm] * 3
    t = np.arange(STEPS) * np.float32(dt)
    f0, spread = 15e9, 20e-12
    pw = (np.sin(2 * np.pi * f0 * (t - 3 * spread)) *
          np.exp(-((t - 3 * spread) / spread) ** 2)).astype(np.float32)
    probes = np.stack([rng.integers(1, d - 2 * PML - 1, 5) for d in DIMS], axis=1).astype(np.int32)
    return dict(fr=np.float32([f0, dx, dt]), td=np.int32([STEPS, I, J, K, 5]), eps=eps, sig=sig,
                mu=mu, sm=sm, pw=pw, probes=np.asfortranarray(probes))


def _ready(api, inp, mode, magnetic=True):
    P = api("CreateSimulation")
    api("SetParams", P, np.float64([PML, W, 3, 1, 0.08, 1, 0.8, 0]))
    api("SetConst", P, inp["fr"], inp["td"])
    api("SetAntennaLocations", P, inp["probes"])
    for f in (1, 2, 3):
        api("UpdateMaterial", P, np.int32(f), inp["sig"])
    for f in (4, 5, 6):
        api("UpdateMaterial", P, np.int32(f), inp["eps"])
    api("ReadySimulation", P)
    if magnetic:
        api("SetMagnetic", P, *inp["mu"], *inp["sm"])
    if mode == 5:
        api("SetIncidence", P, np.float64(ANG))
    api("Init1D", P, np.float32(1.0), inp["pw"])
    return P


def _fields(api, P):
    n = int(np.prod(DIMS))
    return [api("OutputVis", P, np.uint32(n), np.int32(f)) for f in range(1, 7)]


def _oracle(inp, prec, mode):
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
    o.set_magnetic(inp["mu"], inp["sm"])
    if mode == 5:
        o.set_incidence(*ANG)
    o.init_1d(1.0, inp["pw"])
    o.update_cuda()
    o.reset_field_all()
    for n in range(STEPS):
        o.step(n, mode)
    return o


@pytest.mark.parametrize("mode,per_cell", [(3, False), (5, False), (1, True)])
def test_magnetic_equals_oracle(mode, per_cell):
    from maxwell_solver_gb300 import info, simFDTD

    inp = _inputs(per_cell)
    P = _ready(simFDTD, inp, mode)
    assert info(P)["hcoef_mode"] == (1 if per_cell else 2)
    simFDTD("StepN", P, np.int32([0, STEPS, mode]))
    got = _fields(simFDTD, P)
    probes = simFDTD("OutputProbes", P, np.uint32(STEPS * 5 * 6))
    simFDTD("DeleteSimulation", P)
    o32 = _oracle(inp, "f32", mode)
    for a, name in zip(got, FIELDS):
        np.testing.assert_array_equal(a, o32.field(name), err_msg=name)
    np.testing.assert_array_equal(probes, o32.array("probes"))
    o64 = _oracle(inp, "f64", mode)
    for fam in (slice(0, 3), slice(3, 6)):  # relative L2 per family <= 1e-5
        mine = np.concatenate([g.astype(np.float64) for g in got[fam]])
        ref = np.concatenate([np.asarray(o64.field(n), np.float64) for n in FIELDS[fam]])
        assert np.linalg.norm(mine - ref) / np.linalg.norm(ref) <= 1e-5
    assert np.abs(got[4]).max() > 1e-4


def test_magnetic_per_op_calls_equal_step_n(mex):
    from maxwell_solver_gb300 import simFDTD

    inp = _inputs(seed=32)
    P = _ready(simFDTD, inp, 3)
    simFDTD("StepN", P, np.int32([0, STEPS, 3]))
    want = _fields(simFDTD, P)
    Q = _ready(mex, inp, 3)
    for n in range(STEPS):
        tm = np.int32([n, 3])
        mex("UpdateH_All", Q)
        mex("UpdateH_PlaneWave", Q, tm)
        mex("UpdateH_PML", Q)
        mex("UpdateE_All", Q)
        mex("UpdateE_PlaneWave", Q, tm)
        mex("UpdateE_PML", Q)
    for a, b in zip(_fields(mex, Q), want):
        np.testing.assert_array_equal(a, b)
    simFDTD("DeleteSimulation", P)
    mex("DeleteSimulation", Q)


@pytest.mark.parametrize("mode", [3, 5])
def test_unit_mu_reproduces_the_default_update(mode):
    from maxwell_solver_gb300 import simFDTD

    inp = _inputs(seed=33)
    n = int(np.prod(DIMS))
    inp["mu"] = [np.ones(n, np.float32)] * 3
    inp["sm"] = [np.zeros(n, np.float32)] * 3
    out = []
    for magnetic in (True, False):
        P = _ready(simFDTD, inp, mode, magnetic)
        simFDTD("StepN", P, np.int32([0, STEPS, mode]))
        out.append(_fields(simFDTD, P))
        simFDTD("DeleteSimulation", P)
    for a, b, name in zip(out[0], out[1], FIELDS):
        np.testing.assert_array_equal(a, b, err_msg=name)


def test_magnetic_refusals():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD
    from maxwell_solver_gb300.batch import Batch

    inp = _inputs(seed=34)
    n = int(np.prod(DIMS))
    P = simFDTD("CreateSimulation")
    simFDTD("SetConst", P, inp["fr"], inp["td"])
    with pytest.raises(SimFDTDError) as e:  # before ReadySimulation
        simFDTD("SetMagnetic", P, *inp["mu"])
    assert e.value.identifier == "simFDTD:InvalidState"
    simFDTD("DeleteSimulation", P)
    P = _ready(simFDTD, inp, 3)
    bad = np.ones(n, np.float32)
    bad[7] = 0.0
    with pytest.raises(SimFDTDError) as e:  # mu_r must be positive
        simFDTD("SetMagnetic", P, bad, bad, bad)
    assert e.value.identifier == "simFDTD:InvalidInput"
    with Batch() as b:  # the batched kernels use the scalar coefficients
        with pytest.raises(SimFDTDError) as e:
            b.add(P, 0, STEPS, 3)
    assert "uniform H coefficients" in str(e.value)
    simFDTD("DeleteSimulation", P)
