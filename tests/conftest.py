import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


MEX_SRC = os.path.join(ROOT, "maxwell_solver_gb300", "csrc", "mex", "simFDTD_mex.c")
STUB_DIR = os.path.join(ROOT, "tests", "mexstub")
TEST_BUILD = os.path.join(ROOT, "tests", "_build")


def build_mex_shim() -> str:
    """Compiles the drop-in mexFunction against the MEX stub and links it to
    libfdtd_gb300.so (tests only: MATLAB is not installed)."""
    import subprocess

    from maxwell_solver_gb300.build import LIB, LIB_DIR, build

    build()
    os.makedirs(TEST_BUILD, exist_ok=True)
    out = os.path.join(TEST_BUILD, "libsimfdtd_mexstub.so")
    deps = [MEX_SRC, os.path.join(STUB_DIR, "mexstub.c"), os.path.join(STUB_DIR, "mex.h"), LIB]
    if not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out) for d in deps):
        tmp = out + f".tmp{os.getpid()}"
        subprocess.run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-o", tmp, MEX_SRC,
                        os.path.join(STUB_DIR, "mexstub.c"), f"-I{STUB_DIR}",
                        f"-I{os.path.join(ROOT, 'include')}", f"-L{LIB_DIR}", "-lfdtd_gb300",
                        f"-Wl,-rpath,{LIB_DIR}"], check=True)
        os.replace(tmp, out)
    return out


@pytest.fixture(scope="session")
def mex():
    from mexstub.mexdrv import MexDriver

    return MexDriver(build_mex_shim(), "mexFunction")


@pytest.fixture(scope="session")
def native_lib():
    from maxwell_solver_gb300 import _native
    from maxwell_solver_gb300.build import build

    build()
    return _native.load()
