"""The reference's own CUDA kernels, run on this GPU -- TEST INFRASTRUCTURE.

oracle/ref_gpu_build.py compiles the reference's kernel header (src/gpu.h)
for sm_103a into oracle/_ref/ref_gpu.cubin (the reference's nvcc defaults:
multiply-add contraction on) and ref_gpu_nofma.cubin (contraction off).
RefGPU loads one of them through the CUDA driver API and drives the
kernels the way the reference's simulation class does: the host set-up
(SetConst, UpdateMaterial, ReadySimulation, Init1D, UpdateCuda) is the CPU
oracle's restatement of src/simulation.h:79-131, 134-254, 640-979 and
1097-1127, whose arrays are uploaded as they are; every step op launches
the reference's kernels with the reference's launch shapes and arguments
(src/simulation.h:256-286, 330-570; 1024 threads per block, 32 x 32 blocks
for the TF/SF faces).  RefGPU is called like simFDTD (op string, handle,
arguments), so tests/scenarios.run_mex drives it unchanged.

Used by tests/test_reference_gpu.py only: parity of the library against
the reference's own kernels on the same GPU, and their step time.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref")
NT = 1024  # NumThreads, src/simulation.h:18
BS = 32  # block_size, src/simulation.h:75


def unavailable() -> str | None:
    """Why the reference kernels cannot run here (None: they can)."""
    for f in ("ref_gpu.cubin", "ref_gpu_nofma.cubin", "ref_gpu_names.json"):
        if not os.path.isfile(os.path.join(REF, f)):
            return f"oracle/_ref/{f} missing (python oracle/ref_gpu_build.py REFERENCE_ROOT)"
    try:
        import torch
    except ImportError:
        return "torch missing"
    if not torch.cuda.is_available():
        return "no GPU"
    return None


class _Module:
    """One cubin loaded into the current (torch's primary) context."""

    def __init__(self, path: str, names: dict):
        import torch

        torch.zeros(1, device="cuda")  # the primary context is current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                                ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.cu.cuModuleUnload.argtypes = [ctypes.c_void_p]
        with open(path, "rb") as f:
            self._image = f.read()
        self.mod = ctypes.c_void_p()
        self._ok(self.cu.cuModuleLoadData(ctypes.byref(self.mod), self._image), "load " + path)
        self.fn = {}
        for k, low in names.items():
            f = ctypes.c_void_p()
            self._ok(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, low.encode()), k)
            self.fn[k] = f

    def _ok(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"CUDA driver error {rc}: {what}")

    def launch(self, name, grid, block, args, stream):
        """args: ctypes scalars (c_void_p pointers, c_float, c_size_t)."""
        gx, gy = (grid, 1) if isinstance(grid, int) else grid
        bx, by = (block, 1) if isinstance(block, int) else block
        if gx <= 0 or gy <= 0:
            return
        params = (ctypes.c_void_p * len(args))(
            *[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self._ok(self.cu.cuLaunchKernel(self.fn[name], gx, gy, 1, bx, by, 1, 0, stream, params,
                                        None), name)

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = ctypes.c_void_p()


class RefGPU:
    """A simFDTD-shaped driver over the reference's kernels (one handle)."""

    def __init__(self, fma: bool = True, params: dict | None = None):
        import torch

        from oracle import OracleSim

        self.m = None
        self.load(fma)
        self.torch = torch
        self.o = OracleSim("f32")
        if params:
            self.o.set_params(**params)
        self.stream = torch.cuda.current_stream().cuda_stream
        self.d = {}
        self.src = None

    def load(self, fma: bool):
        """Switches to the build with (True) or without multiply-add
        contraction; the fields and set-up stay as they are."""
        with open(os.path.join(REF, "ref_gpu_names.json")) as f:
            names = json.load(f)["kernels"]
        if self.m is not None:
            self.m.close()
        self.m = _Module(os.path.join(REF, "ref_gpu.cubin" if fma else "ref_gpu_nofma.cubin"),
                         names)

    # ------------------------------------------------------------ set-up
    def _up(self, name, arr):
        t = self.torch
        self.d[name] = t.from_numpy(np.ascontiguousarray(arr, dtype=np.float32)).to("cuda")

    def _zeros(self, name, n):
        self.d[name] = self.torch.zeros(int(n), dtype=self.torch.float32, device="cuda")

    def _upload_coefficients(self):
        for c in ("Cexe", "Ceye", "Ceze", "Cexh", "Ceyh", "Cezh"):
            self._up(c, self.o.field(c))
        for a in ("b_E", "c_E", "b_H", "c_H"):
            self._up(a, self.o.array(a))

    def _allocate(self):
        I, J, K = self.o.shape
        p = self.o.dim("p")
        for f in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
            self._zeros(f, I * J * K)
        for nm in ("psi_Exy", "psi_Ezy", "psi_Hxy", "psi_Hzy"):
            self._zeros(nm, 2 * I * p * K)
        for nm in ("psi_Exz", "psi_Eyz", "psi_Hxz", "psi_Hyz"):
            self._zeros(nm, 2 * I * J * p)
        for nm in ("psi_Eyx", "psi_Ezx", "psi_Hyx", "psi_Hzx"):
            self._zeros(nm, 2 * p * J * K)

    # -------------------------------------------------------- arguments
    def _p(self, name):
        return ctypes.c_void_p(self.d[name].data_ptr())

    @staticmethod
    def _f(x):
        return ctypes.c_float(float(x))

    @staticmethod
    def _z(x):
        return ctypes.c_size_t(int(x))

    def _dims(self):
        I, J, K = self.o.shape
        return [self._z(I), self._z(J), self._z(K)]

    def _box(self):
        return [self._z(self.o.dim(n)) for n in ("i0", "i1", "j0", "j1", "k0", "k1")]

    # ---------------------------------------------------------- step ops
    def update_h(self):
        I, J, K = self.o.shape
        o = self.o
        self.m.launch("GPU_updateH", (I * J * K + NT - 1) // NT, NT,
                      [self._p(f) for f in ("Hx", "Hy", "Hz", "Ex", "Ey", "Ez")]
                      + [self._f(o.scalar("Chh")), self._f(o.scalar("Che"))] + self._dims()
                      + [self._z(I * J)], self.stream)

    def update_e(self):
        I, J, K = self.o.shape
        self.m.launch("GPU_updateE", (I * J * K + NT - 1) // NT, NT,
                      [self._p(f) for f in ("Ex", "Ey", "Ez", "Cexe", "Cexh", "Ceye", "Ceyh",
                                            "Ceze", "Cezh", "Hx", "Hy", "Hz")]
                      + self._dims() + [self._z(I * J)], self.stream)

    def _grids(self):
        I, J, K = self.o.shape
        p = self.o.dim("p")
        g = lambda n: (2 * n + NT - 1) // NT  # noqa: E731
        return g(p * J * K), g(I * p * K), g(I * J * p)  # gridsize_x / _y / _z

    def update_h_pml(self):
        I, J, K = self.o.shape
        gx, gy, gz = self._grids()
        che, dx, p = self._f(self.o.scalar("Che")), self._f(self.delX), self._z(self.o.dim("p"))
        tail = [self._p("b_H"), self._p("c_H"), p, che, dx] + self._dims() + [self._z(I * J)]
        self.m.launch("GPU_updateHPmlY", gy, NT, [self._p(f) for f in (
            "Hx", "Hz", "Ex", "Ez", "psi_Hxy", "psi_Hzy")] + tail, self.stream)
        self.m.launch("GPU_updateHPmlX", gx, NT, [self._p(f) for f in (
            "Hy", "Hz", "Ey", "Ez", "psi_Hyx", "psi_Hzx")] + tail, self.stream)
        self.m.launch("GPU_updateHPmlZ", gz, NT, [self._p(f) for f in (
            "Hx", "Hy", "Ex", "Ey", "psi_Hxz", "psi_Hyz")] + tail, self.stream)

    def update_e_pml(self):
        I, J, K = self.o.shape
        gx, gy, gz = self._grids()
        dx, p = self._f(self.delX), self._z(self.o.dim("p"))
        bc = [self._p("b_E"), self._p("c_E")]
        tail = [dx, p] + self._dims() + [self._z(I * J)]
        self.m.launch("GPU_updateEPmlY", gy, NT, [self._p(f) for f in (
            "Hx", "Hz", "Ex", "Ez", "psi_Exy", "psi_Ezy")] + bc
            + [self._p("Cexh"), self._p("Cezh")] + tail, self.stream)
        self.m.launch("GPU_updateEPmlZ", gz, NT, [self._p(f) for f in (
            "Hx", "Hy", "Ex", "Ey", "psi_Exz", "psi_Eyz")] + bc
            + [self._p("Cexh"), self._p("Ceyh")] + tail, self.stream)
        self.m.launch("GPU_updateEPmlX", gx, NT, [self._p(f) for f in (
            "Hy", "Hz", "Ey", "Ez", "psi_Eyx", "psi_Ezx")] + bc
            + [self._p("Ceyh"), self._p("Cezh")] + tail, self.stream)

    def _pw(self, name, grid, block, field, src1d, c, coef):
        self.m.launch(name, grid, block, [self._p(field), self._p(src1d), self._f(c), coef]
                      + self._dims() + self._box() + [self._z(self._time)], self.stream)

    def update_h_planewave(self, n, mode):
        I, J, K = self.o.shape
        s1 = self.o.dim("size1d")
        che = self._f(self.o.scalar("Che"))
        b2 = (BS, BS)
        i0, i1, j0, j1, k0, k1 = (self.o.dim(x) for x in ("i0", "i1", "j0", "j1", "k0", "k1"))
        if mode == 1:  # ZY, src/simulation.h:481-492
            self._time = n * s1 + s1 - K
            nbs = ((i1 - i0 + 1) * (j1 - 1 - j0 + 1) + NT - 1) // NT
            self._pw("GPU_updateHx_PlaneWaveZ_Y", nbs, NT, "Hx", "Ez_1D", 1.0, che)
            nbs = ((j1 - 1 - j0 + 1) * (k1 - k0 + 1) + NT - 1) // NT
            self._pw("GPU_updateHz_PlaneWaveZ_Y", nbs, NT, "Hz", "Ez_1D", 1.0, che)
        elif mode == 2:  # ZX, :468-480
            self._time = n * s1 + s1 - K
            self._pw("GPU_updateHy_PlaneWaveZ_X", (I // BS + 1, J // BS + 1), b2, "Hy", "Ez_1D",
                     1.0, che)
            self._pw("GPU_updateHz_PlaneWaveZ_X", (I // BS + 1, K // BS + 1), b2, "Hz", "Ez_1D",
                     1.0, che)
        elif mode == 3:  # XZ, :434-445
            self._time = n * s1 + s1 - I
            self._pw("GPU_updateHx_PlaneWaveX_Z", (I // BS + 1, K // BS + 1), b2, "Hx", "Ez_1D",
                     1.0, che)
            self._pw("GPU_updateHy_PlaneWaveX_Z", (J // BS + 1, K // BS + 1), b2, "Hy", "Ez_1D",
                     1.0, che)
        elif mode == 4:  # XY, :421-433
            self._time = n * s1 + s1 - I
            self._pw("GPU_updateHx_PlaneWaveX_Y", (I // BS + 1, J // BS + 1), b2, "Hx",
                     "E_inv_1D", 1.0, che)
            self._pw("GPU_updateHz_PlaneWaveX_Y", (J // BS + 1, K // BS + 1), b2, "Hz",
                     "E_inv_1D", 1.0, che)

    def update_e_planewave(self, n, mode):
        I, J, K = self.o.shape
        s1 = self.o.dim("size1d")
        b2 = (BS, BS)
        if mode == 1:  # ZY, :558-570
            self._time = n * s1 + s1 - K
            self._pw("GPU_updateEy_PlaneWaveZ_Y", (I // BS + 1, J // BS + 1), b2, "Ey", "Hy_1D",
                     1.0, self._p("Ceyh"))
            self._pw("GPU_updateEz_PlaneWaveZ_Y", (I // BS + 1, K // BS + 1), b2, "Ez", "Hy_1D",
                     1.0, self._p("Cezh"))
        elif mode == 2:  # ZX, :545-557
            self._time = n * s1 + s1 - K
            self._pw("GPU_updateEx_PlaneWaveZ_X", (I // BS + 1, J // BS + 1), b2, "Ex", "Hy_1D",
                     -1.0, self._p("Cexh"))
            self._pw("GPU_updateEz_PlaneWaveZ_X", (J // BS + 1, K // BS + 1), b2, "Ez", "Hy_1D",
                     -1.0, self._p("Cezh"))
        elif mode == 3:  # XZ, :506-518
            self._time = n * s1 + s1 - I
            self._pw("GPU_updateEx_PlaneWaveX_Z", (I // BS + 1, J // BS + 1), b2, "Ex", "Hy_1D",
                     1.0, self._p("Cexh"))
            self._pw("GPU_updateEz_PlaneWaveX_Z", (J // BS + 1, K // BS + 1), b2, "Ez", "Hy_1D",
                     1.0, self._p("Cezh"))
        elif mode == 4:  # XY, :493-505
            self._time = n * s1 + s1 - I
            self._pw("GPU_updateEx_PlaneWaveX_Y", (I // BS + 1, K // BS + 1), b2, "Ex",
                     "H_inv_1D", -1.0, self._p("Cexh"))
            self._pw("GPU_updateEy_PlaneWaveX_Y", (J // BS + 1, K // BS + 1), b2, "Ey",
                     "H_inv_1D", -1.0, self._p("Ceyh"))

    def add_currents(self, n, mode, box):
        I, J, K = self.o.shape
        i0, i1, j0, j1, k0, k1 = (int(x) for x in box)
        total = (i1 - i0 + 1) * (j1 - j0 + 1) * (k1 - k0 + 1)
        f, ce, ch = {1: ("Ex", "Cexe", "Cexh"), 2: ("Ey", "Ceye", "Ceyh"),
                     3: ("Ez", "Ceze", "Cezh")}[mode]
        self.m.launch("AddSource_GPU_3D_1DThread", (total + NT - 1) // NT, NT,
                      [self._p(f), self._p(ce), self._p(ch), self._f(self.delX)] + self._dims()
                      + [self._z(x) for x in (i0, i1, j0, j1, k0, k1)]
                      + [self._f(self.src[n])], self.stream)

    def step(self, n, mode, ops=("H", "HPW", "HPML", "E", "EPW", "EPML")):
        for op in ops:
            if op == "H":
                self.update_h()
            elif op == "HPW":
                self.update_h_planewave(n, mode)
            elif op == "HPML":
                self.update_h_pml()
            elif op == "E":
                self.update_e()
            elif op == "EPW":
                self.update_e_planewave(n, mode)
            elif op == "EPML":
                self.update_e_pml()

    def field(self, name) -> np.ndarray:
        self.torch.cuda.synchronize()
        return self.d[name].cpu().numpy()

    # ----------------------------------------------- simFDTD-shaped calls
    def __call__(self, op, P=None, *args):
        o = self.o
        if op == "CreateSimulation":
            return np.uint64(1)
        if op == "SetParams":  # the library's extension op, same order
            v = [float(x) for x in np.asarray(args[0]).ravel()]
            o.set_params(int(v[0]), int(v[1]), *v[2:8])
        elif op == "SetConst":
            o.set_const(args[0], args[1])
            self.delX = float(np.float32(np.asarray(args[0]).ravel()[1]))
        elif op == "SetSource":
            self.src = np.asarray(args[0], dtype=np.float32).ravel()
            o.set_source(args[0])
        elif op == "SetAntennaLocations":
            o.set_antenna_locations(args[0])
        elif op == "UpdateMaterial":
            o.update_material(int(np.asarray(args[0]).ravel()[0]), args[1])
        elif op == "ReadySimulation":
            o.ready_simulation()
            self._allocate()
            self._upload_coefficients()
        elif op == "Init1D":
            o.init_1d(float(np.asarray(args[0]).ravel()[0]), args[1])
            for a in ("Ez_1D", "Hy_1D", "E_inv_1D", "H_inv_1D"):
                self._up(a, o.array(a))
        elif op == "UpdateCuda":
            o.update_cuda()
            self._upload_coefficients()
        elif op == "ResetFieldAll":
            for k, t in self.d.items():
                if k in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz") or k.startswith("psi_"):
                    t.zero_()
        elif op == "UpdateH_All":
            self.update_h()
        elif op == "UpdateE_All":
            self.update_e()
        elif op == "UpdateH_PML":
            self.update_h_pml()
        elif op == "UpdateE_PML":
            self.update_e_pml()
        elif op == "UpdateH_PlaneWave":
            n, mode = (int(x) for x in np.asarray(args[0]).ravel()[:2])
            self.update_h_planewave(n, mode)
        elif op == "UpdateE_PlaneWave":
            n, mode = (int(x) for x in np.asarray(args[0]).ravel()[:2])
            self.update_e_planewave(n, mode)
        elif op == "AddCurrents":
            n, mode = (int(x) for x in np.asarray(args[0]).ravel()[:2])
            self.add_currents(n, mode, np.asarray(args[1]).ravel())
        elif op == "DeleteSimulation":
            self.close()
        else:
            raise ValueError(f"RefGPU: op {op} not driven")
        return None

    def close(self):
        self.d.clear()
        self.m.close()
        self.o.close()
