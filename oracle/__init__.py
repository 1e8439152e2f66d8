"""CPU oracle for the FDTD step loop -- TEST INFRASTRUCTURE ONLY.

``fdtd_oracle.c`` restates the reference (src/simulation.h, src/gpu.h of
enricoballini/maxwell_solver) op by op.  This module compiles it (FP32 and
FP64 builds in one shared object) and wraps it with ctypes.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use it, as the
checker; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libfdtd_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_fdtd.so")
REF_FUNLIB_PATH = os.path.join(HERE, "_ref", "libref_funlib.so")
_SRC = os.path.join(HERE, "fdtd_oracle.c")

# field ids shared with fdtd_oracle.c's OR(field)
FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
COEFS = ("Cexe", "Ceye", "Ceze", "Cexh", "Ceyh", "Cezh")
PSI = ("Exy", "Exz", "Eyx", "Eyz", "Ezx", "Ezy",
       "Hxy", "Hxz", "Hyx", "Hyz", "Hzx", "Hzy")
ARRAYS = ("b_E", "c_E", "b_H", "c_H", "den_ex", "den_hx",
          "Ez_1D", "Hy_1D", "E_inv_1D", "H_inv_1D", "probes", "ob_E", "ob_H")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compiles the FP32 + FP64 oracle into oracle/_build/libfdtd_oracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(_SRC)):
        return LIB_PATH
    objs = []
    for real, suffix in (("float", "f32"), ("double", "f64")):
        obj = os.path.join(BUILD_DIR, f"fdtd_oracle_{suffix}.o")
        subprocess.run(
            ["gcc", "-std=gnu11", "-O3", "-fopenmp", "-ffp-contract=off",
             "-fPIC", "-c", _SRC, f"-DOR_REAL={real}", f"-DOR_SUFFIX={suffix}",
             "-o", obj], check=True)
        objs.append(obj)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run(["gcc", "-shared", "-fopenmp", "-o", tmp, *objs, "-lm"],
                   check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_root(ref_root: str | None = None) -> str | None:
    """The reference checkout: the argument, else $MAXWELL_REF; None when
    neither names a directory holding the reference's sources."""
    root = ref_root or os.environ.get("MAXWELL_REF")
    if not root or not os.path.exists(os.path.join(root, "src", "simulation.h")):
        return None
    return root


def build_reference(ref_root: str | None = None) -> str | None:
    """Builds oracle/_ref/libref_fdtd.so from the reference sources when
    they are present (see reference_root); returns its path or None."""
    root = reference_root(ref_root)
    if root is None:
        return None
    subprocess.run([os.path.join(HERE, "ref_build.sh"), root], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_LIB_PATH


def build_reference_funlib(ref_root: str | None = None) -> str | None:
    """Builds oracle/_ref/libref_funlib.so, the reference's source-waveform
    MEX file (src/cpucode/FunLib.cpp) against the test MEX stand-in, when
    the reference sources are present; returns its path or None."""
    root = reference_root(ref_root)
    if root is None or not os.path.exists(os.path.join(root, "src", "cpucode", "FunLib.cpp")):
        return None
    subprocess.run([os.path.join(HERE, "funlib_build.sh"), root], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_FUNLIB_PATH


def build_reference_gpu(ref_root: str | None = None) -> str | None:
    """Builds oracle/_ref/ref_gpu.cubin and ref_gpu_nofma.cubin, the
    reference's own kernels (src/gpu.h) for sm_103a through NVRTC, when the
    reference sources are present; returns the directory or None."""
    root = reference_root(ref_root)
    if root is None or not os.path.exists(os.path.join(root, "src", "gpu.h")):
        return None
    subprocess.run([sys.executable, os.path.join(HERE, "ref_gpu_build.py"), root], check=True,
                   stdout=subprocess.DEVNULL)
    return os.path.join(HERE, "_ref")


def _load():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            lib = ctypes.CDLL(LIB_PATH)
            for sfx, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
                P = ctypes.c_void_p
                f = lambda n: getattr(lib, f"ora_{sfx}_{n}")  # noqa: E731
                f("create").restype = P
                f("set_threads").argtypes = [ctypes.c_int]
                f("set_threads").restype = None
                f("threads").restype = ctypes.c_int
                f("destroy").argtypes = [P]
                f("set_params").argtypes = [P, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6
                f("set_const").argtypes = [P, P, P]
                f("set_source").argtypes = [P, P]
                f("update_material").argtypes = [P, ctypes.c_int, P]
                f("set_antenna_locations").argtypes = [P, P]
                f("ready_simulation").argtypes = [P]
                f("init_1d").argtypes = [P, ctypes.c_float, P]
                f("set_incidence").argtypes = [P] + [ctypes.c_double] * 3
                f("set_magnetic").argtypes = [P] * 7
                f("update_cuda").argtypes = [P]
                f("reset_field_all").argtypes = [P]
                for n in ("update_h_all", "update_e_all", "update_h_pml", "update_e_pml"):
                    f(n).argtypes = [P]
                    f(n).restype = None
                for n in ("update_h_planewave", "update_e_planewave", "step"):
                    f(n).argtypes = [P, ctypes.c_int, ctypes.c_int]
                f("add_currents").argtypes = [P, ctypes.c_int, ctypes.c_int, P]
                f("sample_probes").argtypes = [P, ctypes.c_int]
                for n in ("field", "psi", "array"):
                    f(n).argtypes = [P, ctypes.c_int]
                    f(n).restype = ctypes.POINTER(ct)
                f("dim").argtypes = [P, ctypes.c_int]
                f("dim").restype = ctypes.c_longlong
                f("scalar").argtypes = [P, ctypes.c_int]
                f("scalar").restype = ctypes.c_double
            _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> int:
    """Runs the oracle's OpenMP loops on n host threads; returns the count
    in use."""
    lib = _load()
    lib.ora_f32_set_threads(int(n))
    lib.ora_f64_set_threads(int(n))
    return int(lib.ora_f32_threads())


def threads() -> int:
    """OpenMP threads the oracle's loops use."""
    return int(_load().ora_f32_threads())


class OracleSim:
    """One oracle simulation; mirrors the reference's simFDTD op sequence.

    ``precision`` is "f32" (parity oracle) or "f64" (error floor).
    Arrays returned by accessors are copies in the oracle's precision.
    """

    def __init__(self, precision: str = "f32"):
        assert precision in ("f32", "f64")
        self._lib = _load()
        self._p = precision
        self._dt = np.float32 if precision == "f32" else np.float64
        self._h = self._f("create")()
        self._keep = []

    def _f(self, name):
        return getattr(self._lib, f"ora_{self._p}_{name}")

    def close(self):
        if self._h:
            self._f("destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- setup (reference op order) ---
    def set_params(self, pml=10, tfsf_width=15, poly_m=3.0, alpha_m=1.0,
                   alpha_max=0.08, kappa_max=1.0, sig_factor=0.8, r0=0.0):
        rc = self._f("set_params")(self._h, pml, tfsf_width, poly_m, alpha_m,
                                   alpha_max, kappa_max, sig_factor, r0)
        assert rc == 0, rc

    def set_const(self, freq_res, time_dim):
        fr = np.ascontiguousarray(freq_res, dtype=np.float32)
        td = np.ascontiguousarray(time_dim, dtype=np.int32)
        assert self._f("set_const")(self._h, _ptr(fr), _ptr(td)) == 0

    def set_source(self, src):
        a = np.ascontiguousarray(src, dtype=np.float32)
        self._f("set_source")(self._h, _ptr(a))

    def update_material(self, flag, values):
        a = np.ascontiguousarray(values, dtype=np.float32).ravel(order="F")
        self._f("update_material")(self._h, int(flag), _ptr(a))

    def set_antenna_locations(self, loc):
        a = np.ascontiguousarray(np.asarray(loc, dtype=np.int32).ravel(order="F"))
        self._f("set_antenna_locations")(self._h, _ptr(a))

    def ready_simulation(self):
        self._f("ready_simulation")(self._h)

    def set_incidence(self, theta, phi, psi):
        """TF/SF mode 5 (oblique plane wave); before init_1d."""
        assert self._f("set_incidence")(self._h, float(theta), float(phi), float(psi)) == 0

    def set_magnetic(self, mu, sm=None):
        """Per-cell mu_r (and magnetic conductivity) of Hx, Hy, Hz: three
        arrays of I*J*K each; after ready_simulation."""
        m = [np.ascontiguousarray(x, dtype=np.float32).ravel(order="F") for x in mu]
        g = [np.ascontiguousarray(x, dtype=np.float32).ravel(order="F") for x in sm] if sm else None
        ptrs = [_ptr(x) for x in m] + ([_ptr(x) for x in g] if g else [None] * 3)
        assert self._f("set_magnetic")(self._h, *ptrs) == 0

    def init_1d(self, rate, pw):
        a = np.ascontiguousarray(pw, dtype=np.float32)
        self._f("init_1d")(self._h, float(rate), _ptr(a))

    def update_cuda(self):
        self._f("update_cuda")(self._h)

    def reset_field_all(self):
        self._f("reset_field_all")(self._h)

    # --- step ops ---
    def update_h_all(self):
        self._f("update_h_all")(self._h)

    def update_e_all(self):
        self._f("update_e_all")(self._h)

    def update_h_pml(self):
        self._f("update_h_pml")(self._h)

    def update_e_pml(self):
        self._f("update_e_pml")(self._h)

    def update_h_planewave(self, n, mode):
        return self._f("update_h_planewave")(self._h, int(n), int(mode))

    def update_e_planewave(self, n, mode):
        return self._f("update_e_planewave")(self._h, int(n), int(mode))

    def add_currents(self, n, mode, box):
        a = np.ascontiguousarray(box, dtype=np.int32)
        return self._f("add_currents")(self._h, int(n), int(mode), _ptr(a))

    def sample_probes(self, n):
        return self._f("sample_probes")(self._h, int(n))

    def step(self, n, mode):
        self._f("step")(self._h, int(n), int(mode))

    # --- readout ---
    def dim(self, which):
        names = ("I", "J", "K", "T", "numAnt", "p", "size1d",
                 "i0", "i1", "j0", "j1", "k0", "k1", "ob_w")
        return int(self._f("dim")(self._h, names.index(which)))

    @property
    def shape(self):
        return (self.dim("I"), self.dim("J"), self.dim("K"))

    def _copy(self, ptr, n):
        if not ptr or n == 0:
            return None
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

    def field(self, name):
        """Flat x-fastest copy of a field / coefficient / material array."""
        ijk = int(np.prod(self.shape))
        names = FIELDS + COEFS + ("sig_x", "sig_y", "sig_z", "eps_x", "eps_y", "eps_z")
        return self._copy(self._f("field")(self._h, names.index(name)), ijk)

    def psi(self, name):
        I, J, K = self.shape
        p = self.dim("p")
        n = {"y": I * 2 * p * K, "z": I * J * 2 * p, "x": 2 * p * J * K}[name[2]]
        return self._copy(self._f("psi")(self._h, PSI.index(name)), n)

    def array(self, name):
        I = self.dim("I")
        p = self.dim("p")
        T = self.dim("T")
        s1 = self.dim("size1d")
        n = {"b_E": 2 * p, "c_E": 2 * p, "b_H": 2 * p, "c_H": 2 * p,
             "den_ex": I, "den_hx": I, "Ez_1D": T * s1, "Hy_1D": T * s1,
             "E_inv_1D": T * s1, "H_inv_1D": T * s1,
             "probes": T * self.dim("numAnt") * 6,
             "ob_E": T * max(self.dim("ob_w"), 0), "ob_H": T * max(self.dim("ob_w"), 0)}[name]
        return self._copy(self._f("array")(self._h, ARRAYS.index(name)), n)

    def scalar(self, name):
        return float(self._f("scalar")(self._h, ("Chh", "Che", "sig_max", "Ceh_1D").index(name)))
