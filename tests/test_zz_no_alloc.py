"""GPU test of the allocation-free entry point fdtd_index_coefficients_static.

That entry point exists for callers that cannot allocate device memory:
applications that route all device memory through their own pool or a
fixed budget, and loops that must not stall other streams with the
device-wide synchronisation cudaMalloc/cudaFree imply.  It builds the same
per-cell material ids and coefficient table as ReadySimulation, with its
scratch in a static device array instead of allocated memory.

The test feeds it the E coefficients of two different grids, one call after
the other (the second call must not see the first call's leftovers), and
checks each result against what the existing ReadySimulation path built for
the same materials: same number of ids, same table (bit for bit, which is
inside the 1e-5 relative-L2 tolerance of the parity tests), and ids that map
every cell back to its own six coefficients.  It also checks that sizes
beyond the static limit are refused.  This file sorts last so that a failure
here never hides the other tests; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from scenarios import by_name, run_mex, run_oracle

pytestmark = pytest.mark.gpu

COEFS = ("Cexe", "Ceye", "Ceze", "Cexh", "Ceyh", "Cezh")
REL_L2_TOL = 1e-5


def _reference_result(name):
    """Material count and table from the existing path (ReadySimulation),
    and the six coefficient arrays of the same grid from the oracle."""
    from maxwell_solver_gb300 import get_table, info, simFDTD

    sc = by_name(name)
    sc0 = type(sc)(**{**sc.__dict__, "steps": 0})
    inp = sc.inputs()
    P = run_mex(simFDTD, sc0, inp)
    inf = info(P)
    assert inf["coef_mode"] == 1
    table = get_table(P, "materials")
    simFDTD("DeleteSimulation", P)
    o = run_oracle(sc0, "f32", inp=inp)
    ce = [o.field(c) for c in COEFS]
    return sc.dims, inf["num_materials"], table, ce


def _call_static(lib, dims, ce_dense, max_ids):
    torch = pytest.importorskip("torch")
    I, J, K = dims
    pitch = (I + 7) // 8 * 8
    dev_ce = []
    for a in ce_dense:
        host = np.zeros((K, J, pitch), dtype=np.float32)
        host[:, :, :I] = a.reshape((K, J, I))
        dev_ce.append(torch.from_numpy(host.ravel()).cuda())
    ids = torch.zeros(pitch * J * K, dtype=torch.int16, device="cuda")
    table = torch.full((max_ids * 6,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ptrs = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in dev_ce])
    n = ctypes.c_int32(-1)
    rc = lib.fdtd_index_coefficients_static(ptrs, I, J, K, pitch, ctypes.c_void_p(ids.data_ptr()),
                                            ctypes.c_void_p(table.data_ptr()), max_ids,
                                            ctypes.byref(n), None)
    return rc, n.value, ids.cpu().numpy().view(np.uint16).reshape((K, J, pitch)), table.cpu().numpy()


def _check_against_reference(lib, name):
    dims, n_ref, table_ref, ce = _reference_result(name)
    rc, n, ids, table = _call_static(lib, dims, ce, max_ids=4096)
    assert rc == 0, lib.fdtd_last_error()
    assert n == n_ref and n > 0
    got = table[: 6 * n]
    rel = np.linalg.norm(got.astype(np.float64) - table_ref) / np.linalg.norm(table_ref)
    assert rel <= REL_L2_TOL
    np.testing.assert_array_equal(got, table_ref)
    I, J, K = dims
    cell_ids = ids[:, :, :I].reshape(-1).astype(np.int64)
    assert cell_ids.max() < n
    rows = got.reshape(n, 6)[cell_ids]
    for c in range(6):
        np.testing.assert_array_equal(rows[:, c], ce[c], err_msg=COEFS[c])


def test_static_indexing_matches_ready_simulation_twice(native_lib):
    # two calls in a row on different grids: the shared scratch is reused
    _check_against_reference(native_lib, "mode1_spheres")
    _check_against_reference(native_lib, "mode2_layers")


def test_static_indexing_rejects_sizes_beyond_its_limit(native_lib):
    dims, _, _, ce = _reference_result("mode1_spheres")
    rc, n, _, _ = _call_static(native_lib, dims, ce, max_ids=40000)
    assert rc == 2 and n == 0
    assert b"32768" in native_lib.fdtd_last_error()
    # more distinct tuples than max_ids: refused, not truncated
    rng = np.random.default_rng(3)
    ce_many = [a.copy() for a in ce]
    ce_many[0] = (0.5 + rng.random(ce[0].size)).astype(np.float32)
    rc, n, _, _ = _call_static(native_lib, dims, ce_many, max_ids=64)
    assert rc == 7 and n == 0
    # and the scratch is usable again afterwards
    _check_against_reference(native_lib, "mode4_spheres")
