"""Seeded FDTD scenarios shared by the golden-vector generator and the tests.

Each scenario is a reference-reachable use of the simFDTD op sequence
(CPML thickness 10, TF/SF inset 15, modes 1-4, current sources), sized so
the CPU oracle finishes in well under a second.  Materials come from a
splitmix64 integer hash, so the same seed gives the same arrays everywhere.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

C0 = 299792458.0

# one step of highfrequency.m:85-91 / GICsimulation.m:119-124
HF_STEP = ("H", "HPW", "HPML", "E", "EPW", "EPML")
GIC_STEP = ("H", "HPML", "E", "EPML", "CUR")


def _splitmix64(state: np.ndarray) -> np.ndarray:
    z = state + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int) -> np.ndarray:
    """n float64 values in [0,1) from a counter-based splitmix64 stream."""
    with np.errstate(over="ignore"):
        ctr = np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x100000001B3)
        bits = _splitmix64(ctr)
    return (bits >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def create_signal(fctr, delT, percentage_bw, num_side_lobes, steps):
    """Sinc-modulated carrier with a cosine window: the waveform of
    src/cpucode/FunLib.cpp:26-44 (float64)."""
    fmaxx = fctr * percentage_bw / 2.0
    spread = 1.0 / (2.0 * delT * fmaxx)
    tto = num_side_lobes * spread
    out = np.zeros(steps)
    for n in range(steps):
        nn = n + 1.0
        v = 0.0
        if nn < 2.0 * tto:
            arg = 2.0 * math.pi * fmaxx * (nn - tto) * delT
            den = 1e-14 if abs(arg) < 1e-14 else arg
            v = math.sin(arg) / den * math.sin(2.0 * math.pi * fctr * (nn - tto) * delT)
        v *= math.cos(((nn - 1.0) / steps) * (math.pi / 2.0))
        out[n] = v
    return out


def gaussian_pulse(steps, t0, width, amp=1.0):
    n = np.arange(steps, dtype=np.float64)
    return amp * np.exp(-((n - t0) ** 2) / (2.0 * width * width))


def materials(kind: str, dims, seed: int, pml: int = 10):
    """Per-component (sigma_x, sigma_y, sigma_z, eps_x, eps_y, eps_z) arrays,
    float32, shaped (I, J, K) (x fastest when flattened in F order)."""
    I, J, K = dims
    eps = np.ones(dims, dtype=np.float64)
    sig = np.zeros(dims, dtype=np.float64)
    if kind == "vacuum":
        pass
    elif kind == "spheres":
        u = uniform(seed, 64)
        ii, jj, kk = np.meshgrid(np.arange(I) + 0.5, np.arange(J) + 0.5,
                                 np.arange(K) + 0.5, indexing="ij")
        for s in range(4):
            cx = pml + 2 + u[8 * s + 0] * (I - 2 * pml - 4)
            cy = pml + 2 + u[8 * s + 1] * (J - 2 * pml - 4)
            cz = pml + 2 + u[8 * s + 2] * (K - 2 * pml - 4)
            r = 2.0 + u[8 * s + 3] * 4.0
            inside = (ii - cx) ** 2 + (jj - cy) ** 2 + (kk - cz) ** 2 <= r * r
            eps[inside] = 1.5 + u[8 * s + 4] * 8.5
            sig[inside] = 10.0 ** (-4.0 + 4.0 * u[8 * s + 5])
    elif kind == "layers":
        u = uniform(seed, 16)
        z = K // 2
        for layer in range(3):
            t = 2 + int(u[3 * layer] * 5)
            e = 5.0 + u[3 * layer + 1] * 25.0
            s = 10.0 ** (-4.0 + 4.0 * u[3 * layer + 2])
            lo = max(0, z - t)
            eps[:, :, lo:z] = e
            sig[:, :, lo:z] = s
            z = lo
        eps[:, :, :z] = eps[:, :, z:z + 1] if z < K else eps[:, :, :z]
        sig[:, :, :z] = sig[:, :, z:z + 1] if z < K else sig[:, :, :z]
    else:
        raise ValueError(kind)
    out = {}
    for a in range(3):
        out[1 + a] = sig.astype(np.float32)
        out[4 + a] = eps.astype(np.float32)
    # anisotropy: scale sigma_y / eps_z slightly so the three components differ
    out[2] = (sig * 0.5).astype(np.float32)
    out[6] = (1.0 + (eps - 1.0) * 0.75).astype(np.float32)
    return out


@dataclass(frozen=True)
class Scenario:
    name: str
    dims: tuple
    steps: int
    mode: int = 0                    # TF/SF mode (0: none)
    step_ops: tuple = HF_STEP
    material: str = "vacuum"
    seed: int = 0
    fctr: float = 30e9
    delX: float = 1e-3
    rate: float = 1.0
    cur_mode: int = 0
    cur_box: tuple = ()
    n_probes: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def delT(self):
        return 0.99 * self.delX / (math.sqrt(3.0) * C0)

    def inputs(self):
        I, J, K = self.dims
        T = self.steps
        fr = np.array([self.fctr, self.delX, self.delT], dtype=np.float32)
        td = np.array([T, I, J, K, self.n_probes], dtype=np.int32)
        pw = create_signal(self.fctr, float(fr[2]), 0.5, 1, T).astype(np.float32)
        src = gaussian_pulse(T, T * 0.3, T * 0.08, 1.0).astype(np.float32)
        mats = {f: a.ravel(order="F") for f, a in materials(self.material, self.dims, self.seed).items()}
        probes = None
        if self.n_probes:
            u = uniform(self.seed + 1000, 3 * self.n_probes)
            # probe coordinates relative to the CPML (SetAntennaLocations adds it)
            lim = np.array([I, J, K]) - 2 * 10 - 2
            probes = np.stack([(u[a::3] * lim[a]).astype(np.int32) + 1 for a in range(3)], axis=1)
        return dict(freqRes=fr, TimeDim=td, pw=pw, source=src, mats=mats, probes=probes)


SCENARIOS = (
    Scenario("hf_mode3_vacuum", (40, 36, 34), 80, mode=3),
    Scenario("mode1_spheres", (34, 38, 44), 70, mode=1, material="spheres", seed=11),
    Scenario("mode2_layers", (36, 34, 40), 70, mode=2, material="layers", seed=12),
    Scenario("mode4_spheres", (42, 34, 36), 70, mode=4, material="spheres", seed=13),
    Scenario("gic_currents_x", (40, 44, 36), 80, step_ops=GIC_STEP, material="layers",
             seed=14, cur_mode=1, cur_box=(1, 38, 21, 21, 17, 17)),
    Scenario("curl_only_currents_z", (33, 35, 37), 60, step_ops=("H", "E", "CUR"),
             material="spheres", seed=15, cur_mode=3, cur_box=(15, 17, 16, 16, 10, 25)),
    Scenario("mode3_probes_y_current", (48, 40, 36), 60, mode=3,
             step_ops=HF_STEP + ("CUR",), material="spheres", seed=16, cur_mode=2,
             cur_box=(20, 22, 18, 18, 12, 20), n_probes=5),
)


def by_name(name: str) -> Scenario:
    for s in SCENARIOS:
        if s.name == name:
            return s
    raise KeyError(name)


def run_mex(drv, sc: Scenario, inp=None, on_step=None):
    """Drives a simFDTD mexFunction through the scenario; returns the handle."""
    inp = inp or sc.inputs()
    P = drv("CreateSimulation")
    drv("SetConst", P, inp["freqRes"], inp["TimeDim"])
    drv("SetSource", P, inp["source"])
    if inp["probes"] is not None:
        drv("SetAntennaLocations", P, np.asfortranarray(inp["probes"]).astype(np.int32))
    for flag in range(1, 7):
        drv("UpdateMaterial", P, np.int32(flag), inp["mats"][flag])
    drv("ReadySimulation", P)
    if sc.mode:
        drv("Init1D", P, np.float32(sc.rate), inp["pw"])
    drv("UpdateCuda", P)
    drv("ResetFieldAll", P)
    box = np.array(sc.cur_box, dtype=np.int32) if sc.cur_box else None
    for n in range(sc.steps):
        tm = np.array([n, sc.mode], dtype=np.int32)
        for op in sc.step_ops:
            if op == "H":
                drv("UpdateH_All", P)
            elif op == "HPW":
                drv("UpdateH_PlaneWave", P, tm)
            elif op == "HPML":
                drv("UpdateH_PML", P)
            elif op == "E":
                drv("UpdateE_All", P)
            elif op == "EPW":
                drv("UpdateE_PlaneWave", P, tm)
            elif op == "EPML":
                drv("UpdateE_PML", P)
            elif op == "CUR":
                drv("AddCurrents", P, np.array([n, sc.cur_mode], dtype=np.int32), box)
        if on_step:
            on_step(n, P)
    return P


def run_oracle(sc: Scenario, precision="f32", inp=None, steps=None):
    """Runs the scenario on the CPU oracle; returns the OracleSim."""
    from oracle import OracleSim

    inp = inp or sc.inputs()
    o = OracleSim(precision)
    o.set_const(inp["freqRes"], inp["TimeDim"])
    o.set_source(inp["source"])
    if inp["probes"] is not None:
        o.set_antenna_locations(np.asfortranarray(inp["probes"]))
    for flag in range(1, 7):
        o.update_material(flag, inp["mats"][flag])
    o.ready_simulation()
    if sc.mode:
        o.init_1d(sc.rate, inp["pw"])
    o.update_cuda()
    o.reset_field_all()
    for n in range(sc.steps if steps is None else steps):
        if inp["probes"] is not None and o.dim("numAnt"):
            o.sample_probes(n)  # row n: state at the start of step n
        for op in sc.step_ops:
            if op == "H":
                o.update_h_all()
            elif op == "HPW":
                o.update_h_planewave(n, sc.mode)
            elif op == "HPML":
                o.update_h_pml()
            elif op == "E":
                o.update_e_all()
            elif op == "EPW":
                o.update_e_planewave(n, sc.mode)
            elif op == "EPML":
                o.update_e_pml()
            elif op == "CUR":
                o.add_currents(n, sc.cur_mode, sc.cur_box)
    return o
