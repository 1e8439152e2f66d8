"""Failure isolation and request cancel, with every failure made on the
host: a device allocation that fails (fdtd_inject_fault), a device error
word set as a timed-out pipeline wait would set it (fdtd_inject_device_error),
a request cancelled while queued or while on the device.  Nothing here
faults, traps or stalls the GPU.  In each case the failing handle or request
reports the error and every other one finishes bit-identical to running
alone."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FDTD_ERR_CUDA, FDTD_ERR_OOM, FDTD_ERR_CANCELLED = 5, 6, 8
FAULT_NONE, FAULT_DEVICE_ALLOC = 0, 1


def _lib():
    from maxwell_solver_gb300 import _native

    return _native.load()


def _specs(n, seed=61):
    from test_serve_gpu import _small_specs

    return _small_specs(n, seed=seed)


def _alone(specs):
    from test_serve_gpu import _serve

    res, _ = _serve(specs, [0.0] * len(specs), hbm_budget=16 << 30, one_at_a_time=True)
    return res


def test_device_error_word_fails_that_handle_only():
    """The error word of one handle set from the host: its next
    synchronising call reports FDTD_ERR_CUDA (and clears the word), while a
    second handle stepping beside it ends bit-identical to the oracle."""
    from maxwell_solver_gb300 import simFDTD
    from scenarios import by_name, run_mex, run_oracle

    lib = _lib()
    lib.fdtd_last_error.restype = ctypes.c_char_p
    sc = by_name("hf_mode3_vacuum")
    inp = sc.inputs()
    P1 = run_mex(simFDTD, sc, inp)
    h1 = int(P1[0])
    assert lib.fdtd_inject_device_error(h1, 2) == 0
    # a second handle set up and stepped after the word was set
    P2 = run_mex(simFDTD, sc, inp)
    assert lib.fdtd_synchronize(int(P2[0])) == 0
    assert lib.fdtd_synchronize(h1) == FDTD_ERR_CUDA
    assert b"timed out" in lib.fdtd_last_error()
    assert lib.fdtd_synchronize(h1) == 0  # the word was cleared
    ref = run_oracle(sc, "f32", inp=inp)
    ijk = int(np.prod(sc.dims))
    for f, n in zip(range(1, 7), ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
        np.testing.assert_array_equal(simFDTD("OutputVis", P2, np.uint32(ijk), np.int32(f)),
                                      ref.field(n), err_msg=n)
    for P in (P1, P2):
        simFDTD("DeleteSimulation", P)


@pytest.mark.parametrize("countdown", [1, 4])
def test_injected_allocation_failure_on_a_handle(countdown):
    """An allocation of ReadySimulation fails: the call reports
    FDTD_ERR_OOM, the handle can still be deleted, and a new handle set up
    the same way runs bit-exact."""
    from maxwell_solver_gb300 import SimFDTDError, simFDTD
    from scenarios import by_name, run_mex, run_oracle

    lib = _lib()
    sc = by_name("mode1_spheres")
    inp = sc.inputs()
    P = simFDTD("CreateSimulation")
    simFDTD("SetConst", P, inp["freqRes"], inp["TimeDim"])
    assert lib.fdtd_inject_fault(FAULT_DEVICE_ALLOC, countdown) == 0
    with pytest.raises(SimFDTDError) as e:
        simFDTD("ReadySimulation", P)
    assert "injected" in str(e.value)
    simFDTD("DeleteSimulation", P)
    assert lib.fdtd_inject_fault(FAULT_NONE, 0) == 0
    P = run_mex(simFDTD, sc, inp)
    ref = run_oracle(sc, "f32", inp=inp)
    n = int(np.prod(sc.dims))
    np.testing.assert_array_equal(simFDTD("OutputVis", P, np.uint32(n), np.int32(3)),
                                  ref.field("Ez"))
    simFDTD("DeleteSimulation", P)


def test_injected_allocation_failure_fails_one_request():
    """The third device allocation of the first served request fails: that
    request finishes with FDTD_ERR_OOM, the server goes on, and every other
    request's probes and field equal the one-at-a-time run."""
    from maxwell_solver_gb300 import SimFDTDError
    from maxwell_solver_gb300.serve import Server

    lib = _lib()
    specs = _specs(5)
    alone = _alone(specs[1:])
    with Server(hbm_budget=16 << 30, round_steps=16) as srv:
        assert lib.fdtd_inject_fault(FAULT_DEVICE_ALLOC, 3) == 0
        tickets = [srv.submit(s, n_probes=6, out_field=3) for s in specs]
        with pytest.raises(SimFDTDError) as e:
            srv.result(tickets[0])
        assert "FDTD_ERR_OOM" in str(e.value) and "injected" in str(e.value)
        res = [srv.result(t) for t in tickets[1:]]
        st = srv.stats()
    lib.fdtd_inject_fault(FAULT_NONE, 0)
    assert st["failed"] == 1 and st["completed"] == len(specs) - 1
    for spec, a, b in zip(specs[1:], res, alone):
        np.testing.assert_array_equal(a["field"], b["field"], err_msg=str(spec))
        np.testing.assert_array_equal(a["probes"], b["probes"], err_msg=str(spec))


def test_cancel_queued_and_running_requests():
    """Two requests at a time on the device: a queued request cancelled
    never runs, a running one leaves at the end of its round; both finish
    with FDTD_ERR_CANCELLED and the others equal the one-at-a-time run."""
    from maxwell_solver_gb300 import SimFDTDError
    from maxwell_solver_gb300.serve import Server
    from maxwell_solver_gb300.workloads import GridSpec

    specs = _specs(5, seed=67)
    # a long request that is still running when cancelled
    long = GridSpec((64, 64, 64), 3000, 8, 5, 2, 30e9, 67001)
    order = [specs[0], long, specs[1], specs[2], specs[3], specs[4]]
    keep = [0, 2, 4, 5]
    alone = _alone([order[i] for i in keep])
    with Server(hbm_budget=16 << 30, round_steps=8, max_active=2) as srv:
        tickets = [srv.submit(s, n_probes=6, out_field=3) for s in order]
        assert srv.cancel(tickets[3]) == 0  # queued behind the first two
        srv.wait(tickets[0])
        assert srv.cancel(tickets[1]) == 0  # the long one, on the device
        for i in (1, 3):
            with pytest.raises(SimFDTDError) as e:
                srv.result(tickets[i])
            assert "FDTD_ERR_CANCELLED" in str(e.value)
        res = [srv.result(tickets[i]) for i in keep]
        st = srv.stats()
        assert srv.cancel(tickets[0]) != 0  # released ticket
    assert st["cancelled"] == 2 and st["failed"] == 0 and st["completed"] == len(keep)
    for i, a, b in zip(keep, res, alone):
        np.testing.assert_array_equal(a["field"], b["field"], err_msg=str(order[i]))
        np.testing.assert_array_equal(a["probes"], b["probes"], err_msg=str(order[i]))


def test_cancel_after_finish_is_refused():
    from maxwell_solver_gb300.serve import Server

    spec = _specs(1, seed=71)[0]
    with Server(hbm_budget=16 << 30) as srv:
        t = srv.submit(spec, n_probes=6)
        srv.wait(t)
        assert srv.cancel(t) == 3  # FDTD_ERR_STATE: finished already
        assert srv.result(t)["info"]["status"] == 0
