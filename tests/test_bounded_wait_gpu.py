"""Failure detection without a GPU fault: every pipeline wait of the TMA
kernels is bounded.  The self-check runs that wait, with a short poll limit,
on a barrier nothing completes (it must give up and report it) and on one
the waiting thread completes (it must succeed); the context stays usable
(a simulation steps afterwards and matches the oracle), and the measured
time per poll bounds how long the production limit can take."""
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
    assert 0 < poll.value < 1e6
    assert limit.value < 3e3  # the production limit gives up within seconds
    print(f"poll {poll.value:.1f} ns, production limit {limit.value:.1f} ms")

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
