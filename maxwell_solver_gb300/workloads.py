"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every input (materials, sources, probe
positions) is generated from a seed with the sizes and value distributions
the configurations name.

  c1  64^3, 10-cell CPML, vacuum, TF/SF, 500 steps, 8 probes
  c2  256^3, 12-cell CPML, 40 dielectric/lossy spheres (radius U[4,20],
      eps_r U[1.5,10], sigma log-U[1e-4,1] S/m), TF/SF, 2000 steps, 64 probes
  c3  512x512x448, 16-cell CPML, 6-layer conductive half-space below air
      (thickness U[10,80], sigma log-U[1e-4,1], eps_r U[5,30]), vertical
      incidence, 4000 steps, 256-cell surface probe line

Materials are returned as the six per-component arrays the reference's
UpdateMaterial op takes (sigma_x,y,z, eps_x,y,z), flattened x-fastest.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

C0 = 299792458.0


@dataclass(frozen=True)
class Workload:
    name: str
    dims: tuple          # (I, J, K) including the CPML
    steps: int
    pml: int
    mode: int            # TF/SF mode: the reference's 1..4, or 5 (oblique)
    media: str           # vacuum | spheres | layers
    n_probes: int
    seed: int
    delX: float = 1e-3
    fctr: float = 30e9

    @property
    def angles(self) -> tuple:
        """Mode 5: (theta, phi, psi) in radians, seeded."""
        return incidence_angles(self.seed)

    @property
    def delT(self) -> float:
        return 0.99 * self.delX / (math.sqrt(3.0) * C0)

    @property
    def cells(self) -> int:
        return int(np.prod(self.dims))


def incidence_angles(seed: int) -> tuple:
    """Seeded oblique incidence: theta uniform in [0, pi], phi and the
    polarisation angle psi uniform in [0, 2 pi)."""
    r = np.random.default_rng(np.random.PCG64(seed + 104729))
    return (float(r.uniform(0, math.pi)), float(r.uniform(0, 2 * math.pi)),
            float(r.uniform(0, 2 * math.pi)))


WORKLOADS = {
    "c1": Workload("c1", (64, 64, 64), 500, 10, 3, "vacuum", 8, 0),
    "c2": Workload("c2", (256, 256, 256), 2000, 12, 5, "spheres", 64, 1),
    "c3": Workload("c3", (512, 512, 448), 4000, 16, 1, "layers", 256, 2, delX=5e-3, fctr=1e9),
}


def rng(seed: int) -> np.random.Generator:
    return np.random.default_rng(np.random.PCG64(seed))


def materials(w: Workload):
    """dict flag -> float32 array (F-order flattened), flags 1..6."""
    I, J, K = w.dims
    r = rng(w.seed)
    if w.media == "vacuum":
        eps = np.ones((I, J, K), dtype=np.float32, order="F")
        sig = np.zeros((I, J, K), dtype=np.float32, order="F")
    elif w.media == "spheres":
        eps = np.ones((I, J, K), dtype=np.float32, order="F")
        sig = np.zeros((I, J, K), dtype=np.float32, order="F")
        lo = w.pml + 4
        for _ in range(40):
            rad = r.uniform(4, 20)
            c = [r.uniform(lo + rad, n - lo - rad) for n in (I, J, K)]
            e = np.float32(r.uniform(1.5, 10.0))
            s = np.float32(10.0 ** r.uniform(-4, 0))
            b0 = [max(0, int(math.floor(c[a] - rad))) for a in range(3)]
            b1 = [min(n, int(math.ceil(c[a] + rad)) + 1) for a, n in enumerate((I, J, K))]
            x = np.arange(b0[0], b1[0]) + 0.5 - c[0]
            y = np.arange(b0[1], b1[1]) + 0.5 - c[1]
            z = np.arange(b0[2], b1[2]) + 0.5 - c[2]
            inside = (x[:, None, None] ** 2 + y[None, :, None] ** 2 + z[None, None, :] ** 2) <= rad * rad
            sl = (slice(b0[0], b1[0]), slice(b0[1], b1[1]), slice(b0[2], b1[2]))
            eps[sl][inside] = e
            sig[sl][inside] = s
    elif w.media == "layers":
        eps_z = np.ones(K, dtype=np.float32)
        sig_z = np.zeros(K, dtype=np.float32)
        z = K - w.pml - 2 - int(0.45 * K)  # air above, earth below this plane
        top = z
        for _ in range(6):
            t = int(r.integers(10, 81))
            lo = max(0, top - t)
            eps_z[lo:top] = np.float32(r.uniform(5, 30))
            sig_z[lo:top] = np.float32(10.0 ** r.uniform(-4, 0))
            top = lo
            if top == 0:
                break
        if top > 0:
            eps_z[:top] = eps_z[top]
            sig_z[:top] = sig_z[top]
        eps = np.broadcast_to(eps_z[None, None, :], (I, J, K))
        sig = np.broadcast_to(sig_z[None, None, :], (I, J, K))
    else:
        raise ValueError(w.media)
    e = np.asarray(eps, dtype=np.float32).ravel(order="F")
    s = np.asarray(sig, dtype=np.float32).ravel(order="F")
    return {1: s, 2: s, 3: s, 4: e, 5: e, 6: e}


def sources(w: Workload, steps: int | None = None):
    """(plane-wave waveform, current waveform) float32 of length T."""
    T = w.steps if steps is None else steps
    n = np.arange(T, dtype=np.float64)
    dt = np.float32(w.delT)
    if w.media == "layers":
        # Gaussian-derivative pulse, >= 20 cells per shortest wavelength in air
        fmax = C0 / (20 * w.delX)
        tau = 1.0 / (math.pi * fmax)
        t0 = 4 * tau
        t = n * float(dt)
        pw = -(t - t0) / tau * np.exp(-((t - t0) / tau) ** 2)
    else:
        # Gaussian-modulated sine, f0 = fctr, 10 ps spread
        spread = 10e-12
        t = n * float(dt)
        t0 = 4 * spread
        pw = np.sin(2 * math.pi * w.fctr * (t - t0)) * np.exp(-((t - t0) / spread) ** 2)
    cur = np.exp(-((n - 0.3 * T) ** 2) / (2 * (0.08 * T) ** 2))
    return pw.astype(np.float32), cur.astype(np.float32)


def probe_locations(w: Workload) -> np.ndarray:
    """numAnt x 3 int32 (x, y, z) offsets inside the CPML, as
    SetAntennaLocations takes them."""
    I, J, K = w.dims
    p = w.pml
    if w.media == "layers":
        # surface probe line along x at the air/earth interface
        z = K - w.pml - 2 - int(0.45 * K) - p
        xs = np.linspace(2, I - 2 * p - 3, w.n_probes).astype(np.int32)
        return np.stack([xs, np.full_like(xs, (J - 2 * p) // 2), np.full_like(xs, z)], axis=1)
    r = rng(w.seed + 7)
    lim = np.array([I, J, K]) - 2 * p - 2
    return np.stack([r.integers(1, lim[a], w.n_probes) for a in range(3)], axis=1).astype(np.int32)


def setup(api, w: Workload, steps: int | None = None, params=None):
    """Creates and readies a simulation for the workload through a simFDTD
    style callable (this package's simFDTD or a MEX driver); returns P."""
    T = w.steps if steps is None else steps
    I, J, K = w.dims
    P = api("CreateSimulation")
    # TF/SF box 5 cells inside the CPML (15 for the reference's 10 cells)
    api("SetParams", P, np.float64(params if params is not None
                                   else [w.pml, w.pml + 5, 3, 1, 0.08, 1, 0.8, 0]))
    api("SetConst", P, np.float32([w.fctr, w.delX, w.delT]), np.int32([T, I, J, K, w.n_probes]))
    pw, cur = sources(w, T)
    api("SetSource", P, cur)
    if w.n_probes:
        api("SetAntennaLocations", P, np.asfortranarray(probe_locations(w)))
    for flag, arr in materials(w).items():
        api("UpdateMaterial", P, np.int32(flag), arr)
    api("ReadySimulation", P)
    if w.mode == 5:
        api("SetIncidence", P, np.float64(w.angles))
    api("Init1D", P, np.float32(1.0), pw)
    return P


# ------------------------------------------------------------------ batches

@dataclass(frozen=True)
class GridSpec:
    """One solve of a heterogeneous mix (batched configuration c4 / served c5)."""
    dims: tuple
    steps: int
    pml: int
    mode: int
    n_spheres: int
    fctr: float
    seed: int
    delX: float = 1e-3
    media: str = "spheres"  # or "layers"

    @property
    def angles(self) -> tuple:
        """Mode 5: (theta, phi, psi) in radians, seeded."""
        return incidence_angles(self.seed)

    @property
    def delT(self) -> float:
        return 0.99 * self.delX / (math.sqrt(3.0) * C0)

    @property
    def cells(self) -> int:
        return int(np.prod(self.dims))


def batch_mix(n: int = 256, seed: int = 3):
    """c4: axes uniform-integer 32..128, 8-cell CPML, 0..10 spheres, TF/SF
    plane wave at a random oblique incidence and polarisation (mode 5,
    `incidence_angles`), f0 uniform 10..60 GHz, steps uniform 300..1500."""
    r = rng(seed)
    out = []
    for g in range(n):
        dims = tuple(int(x) for x in r.integers(32, 129, 3))
        steps = int(r.integers(300, 1501))
        r.integers(1, 5)  # (the axis-mode draw of earlier mixes: keeps the sequence)
        out.append(GridSpec(dims, steps, 8, 5, int(r.integers(0, 11)),
                            float(r.uniform(10e9, 60e9)), seed * 1000 + g))
    return out


def serve_mix(n: int = 64, seed: int = 4, max_axis: int = 384, max_steps: int = 4000):
    """c5 requests: cubic-ish grids (a base size log-uniform 48..max_axis,
    each axis within +-15% of it), CPML 8..16 cells, random spheres (oblique
    incidence, mode 5) or layered media (vertical incidence, mode 1), steps
    uniform 200..max_steps, f0 uniform 10..60 GHz."""
    r = rng(seed)
    out = []
    for g in range(n):
        base = math.exp(r.uniform(math.log(48), math.log(max_axis)))
        dims = tuple(int(min(max_axis, max(48, round(base * r.uniform(0.85, 1.15)))))
                     for _ in range(3))
        pml = int(r.integers(8, 17))
        media = "layers" if r.random() < 0.5 else "spheres"
        steps = int(r.integers(200, max_steps + 1))
        r.integers(1, 5)  # (the axis-mode draw of earlier mixes: keeps the sequence)
        mode = 1 if media == "layers" else 5
        out.append(GridSpec(dims, steps, pml, mode, int(r.integers(0, 11)),
                            float(r.uniform(10e9, 60e9)), seed * 1000 + g, media=media))
    return out


SHAPE_SPHERE, SHAPE_LAYER_Z, SHAPE_BOX = 1, 2, 3


def grid_shapes(spec: GridSpec):
    """(bg_eps_r, bg_sigma, rows): the spec's media as shape rows
    [kind, eps_r, sigma, g0..g5] (fdtd_shape), applied in order."""
    I, J, K = spec.dims
    r = rng(spec.seed)
    rows = []
    if spec.media == "layers":  # air above, conductive layers below (config 3 style)
        z = K - spec.pml - 2 - int(0.45 * K)
        top = z
        e = s = None
        for _ in range(6):
            t = int(r.integers(10, 81))
            lo = max(0, top - t)
            e = np.float32(r.uniform(5, 30))
            s = np.float32(10.0 ** r.uniform(-4, 0))
            rows.append([SHAPE_LAYER_Z, e, s, lo, top, 0, 0, 0, 0])
            top = lo
            if top == 0:
                break
        if top > 0:  # the deepest layer continues to the bottom
            rows.append([SHAPE_LAYER_Z, e, s, 0, top, 0, 0, 0, 0])
        return 1.0, 0.0, rows
    lo = spec.pml + 2
    room = min(I, J, K) - 2 * lo
    for _ in range(spec.n_spheres):
        rad = min(r.uniform(4, 20), max(room / 2 - 1, 1.0))
        c = [r.uniform(lo + rad, n - lo - rad) for n in (I, J, K)]
        e = np.float32(r.uniform(1.5, 10.0))
        s = np.float32(10.0 ** r.uniform(-4, 0))
        rows.append([SHAPE_SPHERE, e, s, c[0], c[1], c[2], rad, 0, 0])
    return 1.0, 0.0, rows


def rasterize(dims, bg_eps, bg_sig, rows):
    """eps, sigma (float32, F-order flat) of shape rows, with the library's
    tests: sphere ((i+0.5-x)^2 + (j+0.5-y)^2) + (k+0.5-z)^2 <= r*r in
    float64, layer g0 <= k < g1, box g0 <= i < g1 ...; later rows win."""
    I, J, K = dims
    eps = np.full((I, J, K), np.float32(bg_eps), dtype=np.float32, order="F")
    sig = np.full((I, J, K), np.float32(bg_sig), dtype=np.float32, order="F")
    for row in rows:
        kind, e, s = int(row[0]), np.float32(row[1]), np.float32(row[2])
        g = [float(v) for v in row[3:9]]
        if kind == SHAPE_SPHERE:
            c, rad = g[:3], g[3]
            b0 = [max(0, int(math.floor(c[a] - rad))) for a in range(3)]
            b1 = [min(n, int(math.ceil(c[a] + rad)) + 1) for a, n in enumerate((I, J, K))]
            x = np.arange(b0[0], b1[0]) + 0.5 - c[0]
            y = np.arange(b0[1], b1[1]) + 0.5 - c[1]
            z = np.arange(b0[2], b1[2]) + 0.5 - c[2]
            inside = (x[:, None, None] ** 2 + y[None, :, None] ** 2 +
                      z[None, None, :] ** 2) <= rad * rad
            sl = (slice(b0[0], b1[0]), slice(b0[1], b1[1]), slice(b0[2], b1[2]))
            eps[sl][inside] = e
            sig[sl][inside] = s
        else:
            k = np.arange(K, dtype=np.float64)
            mk = (k >= g[0]) & (k < g[1]) if kind == SHAPE_LAYER_Z else \
                (k >= g[4]) & (k < g[5])
            m = np.broadcast_to(mk[None, None, :], (I, J, K))
            if kind == SHAPE_BOX:
                i = np.arange(I, dtype=np.float64)
                j = np.arange(J, dtype=np.float64)
                m = m & ((i >= g[0]) & (i < g[1]))[:, None, None] & \
                    ((j >= g[2]) & (j < g[3]))[None, :, None]
            eps[m] = e
            sig[m] = s
    return eps.ravel(order="F"), sig.ravel(order="F")


def grid_materials(spec: GridSpec):
    """eps, sigma (float32, F-order flat) of the spec's media."""
    return rasterize(spec.dims, *grid_shapes(spec))


def grid_probes(spec: GridSpec, n: int = 8):
    """n probe cells inside the CPML (SetAntennaLocations order: n x 3,
    column-major), seeded by the spec."""
    I, J, K = spec.dims
    r = rng(spec.seed + 7919)
    lim = [I - 2 * spec.pml, J - 2 * spec.pml, K - 2 * spec.pml]
    loc = np.stack([r.integers(1, max(2, lim[a] - 1), n) for a in range(3)], axis=1)
    return np.asfortranarray(loc.astype(np.int32))


def grid_source(spec: GridSpec):
    """Gaussian-modulated sine at the spec's f0 (10 ps spread), float32 [steps]."""
    n = np.arange(spec.steps, dtype=np.float64)
    t = n * float(np.float32(spec.delT))
    spread = 10e-12
    t0 = 4 * spread
    return (np.sin(2 * math.pi * spec.fctr * (t - t0)) *
            np.exp(-((t - t0) / spread) ** 2)).astype(np.float32)


def setup_grid(api, spec: GridSpec):
    """Creates and readies one grid of a mix; returns its handle."""
    I, J, K = spec.dims
    P = api("CreateSimulation")
    api("SetParams", P, np.float64([spec.pml, spec.pml + 5, 3, 1, 0.08, 1, 0.8, 0]))
    api("SetConst", P, np.float32([spec.fctr, spec.delX, spec.delT]),
        np.int32([spec.steps, I, J, K, 0]))
    eps, sig = grid_materials(spec)
    for flag in (1, 2, 3):
        api("UpdateMaterial", P, np.int32(flag), sig)
    for flag in (4, 5, 6):
        api("UpdateMaterial", P, np.int32(flag), eps)
    api("ReadySimulation", P)
    if spec.mode == 5:
        api("SetIncidence", P, np.float64(spec.angles))
    api("Init1D", P, np.float32(1.0), grid_source(spec))
    return P
