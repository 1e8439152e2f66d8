"""Host-side pieces of the batched and served configurations: the shape
rasteriser agrees with a brute-force test of every cell, the request
generators are deterministic and inside their configured ranges, and the
device-memory estimate used for admission grows with the request."""
import ctypes
import math

import numpy as np
import pytest

from maxwell_solver_gb300 import workloads as w


def _brute(dims, bg_e, bg_s, rows):
    I, J, K = dims
    eps = np.full((I, J, K), np.float32(bg_e), np.float32)
    sig = np.full((I, J, K), np.float32(bg_s), np.float32)
    i, j, k = np.meshgrid(np.arange(I), np.arange(J), np.arange(K), indexing="ij")
    for row in rows:
        kind, e, s, g = int(row[0]), np.float32(row[1]), np.float32(row[2]), row[3:9]
        if kind == w.SHAPE_SPHERE:
            x, y, z = (i + 0.5) - g[0], (j + 0.5) - g[1], (k + 0.5) - g[2]
            m = (x * x + y * y) + z * z <= g[3] * g[3]
        elif kind == w.SHAPE_LAYER_Z:
            m = (k >= g[0]) & (k < g[1])
        else:
            m = (i >= g[0]) & (i < g[1]) & (j >= g[2]) & (j < g[3]) & (k >= g[4]) & (k < g[5])
        eps[m] = e
        sig[m] = s
    return eps.ravel(order="F"), sig.ravel(order="F")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_rasterize_matches_every_cell(seed):
    r = np.random.default_rng(seed)
    dims = (23, 31, 19)
    rows = []
    for _ in range(6):
        rows.append([w.SHAPE_SPHERE, r.uniform(1, 9), r.uniform(0, 1),
                     *r.uniform(0, 25, 3), r.uniform(1, 9), 0, 0])
    rows.append([w.SHAPE_LAYER_Z, 4.0, 0.1, 2, 7, 0, 0, 0, 0])
    rows.append([w.SHAPE_BOX, 2.0, 0.3, 3, 11, 5, 9, 1, 18])
    e0, s0 = w.rasterize(dims, 1.0, 0.0, rows)
    e1, s1 = _brute(dims, 1.0, 0.0, rows)
    np.testing.assert_array_equal(e0, e1)
    np.testing.assert_array_equal(s0, s1)


def test_serve_mix_ranges_and_determinism():
    a, b = w.serve_mix(40), w.serve_mix(40)
    assert a == b
    for s in a:
        assert all(48 <= d <= 384 for d in s.dims)
        assert max(s.dims) / min(s.dims) <= 1.15 / 0.85 + 1e-9
        assert 8 <= s.pml <= 16 and 200 <= s.steps <= 4000 and s.mode == (1 if s.media == "layers" else 5)
        assert s.media in ("spheres", "layers")
    assert {s.media for s in a} == {"spheres", "layers"}
    # log-uniform base size: both ends of the range are visited
    sizes = [math.prod(s.dims) ** (1 / 3) for s in w.serve_mix(200)]
    assert min(sizes) < 70 and max(sizes) > 280


def test_layer_shapes_fill_below_the_air():
    spec = w.GridSpec((40, 40, 120), 10, 10, 1, 0, 1e9, 77, media="layers")
    eps, sig = w.grid_materials(spec)
    e = eps.reshape(spec.dims, order="F")
    top = 120 - 10 - 2 - int(0.45 * 120)
    assert (e[:, :, top:] == 1).all() and (e[:, :, :top] >= 5).all()


def test_estimate_device_bytes(native_lib):
    out = ctypes.c_uint64(0)
    assert native_lib.fdtd_estimate_device_bytes(64, 64, 64, 10, 500, 8, ctypes.byref(out)) == 0
    small = out.value
    assert small >= 12 * 64 ** 3 * 4  # fields + coefficients
    assert native_lib.fdtd_estimate_device_bytes(128, 64, 64, 10, 500, 8, ctypes.byref(out)) == 0
    assert out.value > small
    assert native_lib.fdtd_estimate_device_bytes(64, 64, 64, 10, 4000, 8, ctypes.byref(out)) == 0
    assert out.value > small
    assert native_lib.fdtd_estimate_device_bytes(10, 64, 64, 10, 500, 8, ctypes.byref(out)) == 2
