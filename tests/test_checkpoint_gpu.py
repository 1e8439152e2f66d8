"""Checkpoint / resume: a run saved after N steps and resumed in a fresh
handle set up the same way ends bit-identical (fields and probe record) to
the uninterrupted run; a checkpoint of another set-up is refused."""
import numpy as np
import pytest

from scenarios import SCENARIOS, run_mex

pytestmark = pytest.mark.gpu

SC = next(s for s in SCENARIOS if s.name == "mode3_probes_y_current")


def _ready(api, sc, inp):
    return run_mex(api, type(sc)(**{**sc.__dict__, "steps": 0}), inp)


def _steps(api, P, sc, first, count):
    cur = [np.int32([sc.cur_mode, *sc.cur_box])] if sc.cur_mode else []
    api("StepN", P, np.int32([first, count, sc.mode]), *cur)


def _state(api, P, sc):
    n = int(np.prod(sc.dims))
    fields = [api("OutputVis", P, np.uint32(n), np.int32(f)) for f in range(1, 7)]
    probes = api("OutputProbes", P, np.uint32(sc.steps * sc.n_probes * 6))
    return fields, probes


@pytest.mark.parametrize("via", ["python", "mex"])
def test_resume_equals_uninterrupted(via, mex):
    from maxwell_solver_gb300 import simFDTD

    api = simFDTD if via == "python" else mex
    inp = SC.inputs()
    half = SC.steps // 2
    P = _ready(api, SC, inp)
    _steps(api, P, SC, 0, half)
    ck = api("SaveCheckpoint", P)
    assert ck.dtype == np.uint8 and ck.size > 6 * np.prod(SC.dims) * 4
    _steps(api, P, SC, half, SC.steps - half)
    want = _state(api, P, SC)
    Q = _ready(api, SC, inp)
    api("LoadCheckpoint", Q, ck)
    _steps(api, Q, SC, half, SC.steps - half)
    got = _state(api, Q, SC)
    for a, b in zip(got[0], want[0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(got[1], want[1])
    assert np.abs(want[0][2]).max() > 0
    api("DeleteSimulation", P)
    api("DeleteSimulation", Q)


def test_checkpoint_of_other_setup_is_refused():
    from maxwell_solver_gb300 import SimFDTDError, simFDTD

    other = next(s for s in SCENARIOS if s.name == "hf_mode3_vacuum")
    P = _ready(simFDTD, SC, SC.inputs())
    Q = _ready(simFDTD, other, other.inputs())
    ck = simFDTD("SaveCheckpoint", P)
    with pytest.raises(SimFDTDError) as e:
        simFDTD("LoadCheckpoint", Q, ck)
    assert e.value.identifier == "simFDTD:InvalidInput"
    with pytest.raises(SimFDTDError):
        simFDTD("LoadCheckpoint", P, ck[: ck.size // 2])
    simFDTD("DeleteSimulation", P)
    simFDTD("DeleteSimulation", Q)
