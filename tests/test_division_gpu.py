"""The kernels divide by the cell size through a precomputed reciprocal and
one correction step; this checks that, for every float numerator, the GPU
gives bit for bit what its IEEE division a / dx gives (the reference's
operation)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dx", [1e-3, 3.7e-4, 1.0])
def test_division_plan_is_exact_on_gpu(native_lib, dx):
    bad = ctypes.c_uint64(123)
    assert native_lib.fdtd_check_division(ctypes.c_float(dx), ctypes.byref(bad)) == 0, \
        native_lib.fdtd_last_error()
    assert bad.value == 0
