"""Failure detection without a GPU fault: every pipeline wait of the TMA
kernels is bounded by time (the GPU's global timer).  The self-check runs
that wait, with a 1 ms limit, on a barrier nothing completes (it must give
up, after about that long, and report it) and on one the waiting thread
completes (it must succeed); the context stays usable (a simulation steps
afterwards and matches the oracle), and the production limit is 2 s."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_gives_up_and_context_survives():
    from maxwell_solver_gb300 import _native
    from scenarios import by_name, run_mex, run_oracle

    lib = _native.load()
    t, c = ctypes.c_int32(0), ctypes.c_int32(0)
    poll, limit = ctypes.c_double(0), ctypes.c_double(0)
    assert lib.fdtd_check_bounded_wait(ctypes.byref(t), ctypes.byref(c), ctypes.byref(poll),
                                       ctypes.byref(limit)) == 0
    assert t.value == 1  # nothing completed the barrier: the wait gave up
    assert c.value == 1  # completed barrier: the wait returned
    assert 1e6 <= poll.value < 5e7  # gave up after its 1 ms limit (timer read every 32 polls)
    assert limit.value == 2000.0  # the production limit: 2 s
    print(f"check waited {poll.value / 1e6:.3f} ms, production limit {limit.value:.1f} ms")

    from maxwell_solver_gb300 import simFDTD

    sc = by_name("hf_mode3_vacuum")  # the context is still usable
    inp = sc.inputs()
    P = run_mex(simFDTD, sc, inp)
    n = int(np.prod(sc.dims))
    got = [simFDTD("OutputVis", P, np.uint32(n), np.int32(f)) for f in (1, 2, 3)]
    simFDTD("DeleteSimulation", P)
    o = run_oracle(sc, "f32", inp=inp)
    for a, name in zip(got, ("Ex", "Ey", "Ez")):
        np.testing.assert_array_equal(a, o.field(name), err_msg=name)
