"""The compacted CPML X kernels (FDTD_XC=1: the lean curl kernels apply
CPML X themselves, compacted per warp, instead of E's x-slab pass) are not
the default, being slower; they are still bit-exact.  The switch is read
once per process, so the parity and batch tests run again in a child
process with it set."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_compacted_x_kernels_are_exact():
    env = dict(os.environ, FDTD_XC="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu",
                        os.path.join(HERE, "test_parity_gpu.py"),
                        os.path.join(HERE, "test_batch_gpu.py"),
                        os.path.join(HERE, "test_oblique_gpu.py")],
                       env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
