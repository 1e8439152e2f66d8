"""Per-cell magnetic media (fdtd_set_magnetic) in the FP64 oracle, checked
against physics: a plane wave at normal incidence (TF/SF mode 1, along -z)
on a wide block of
- eps_r = 4: reflection coefficient -1/3,
- mu_r = 4: +1/3 (the dual problem: the reflected pulse is the negative of
  the eps_r = 4 one),
- eps_r = mu_r = 4, and a lossy block with sigma_m / mu = sigma / eps: the
  block's impedance equals free space's, so it reflects nothing (up to the
  grid's O((k dx)^2) interface error).
|R(f)| is the spectrum of the reflected pulse (a probe in the scattered-field
region above the block, gated before the block edges' diffraction arrives)
over that of the incident pulse (the vacuum run).  The interface lies on the
H nodes, which take the average mu (the usual control-volume treatment).
(No reference counterpart: the reference's createMu never reaches its H
update; the GPU path is pinned to this oracle bit for bit in
test_magnetic_gpu.py.)"""
import math

import numpy as np
import pytest

oracle = pytest.importorskip("oracle")

NX, NK, PML, W = 128, 80, 8, 13
KLO, KHI = 20, 57           # integer-k nodes inside the block; faces at KLO-1/2, KHI+1/2
STEPS, FDIV = 190, 20       # pulse: Gaussian derivative, f_max = c / (FDIV dx)
DX = 1e-3
C0 = 299792458.0
MU0 = 4e-7 * math.pi
EPS0 = 1 / (C0 * C0 * MU0)
DT = 0.99 * DX / (math.sqrt(3) * C0)


def _profile(v, half, outside=1.0):
    """Values along k on integer nodes (half=False) or k+1/2 nodes."""
    a = np.full(NK, outside, np.float32)
    if not half:
        a[KLO:KHI + 1] = v
    else:
        a[KLO:KHI] = v
        a[KLO - 1] = a[KHI] = (outside + v) / 2
    return a


def _cells(pk):
    f = np.full((NX, NX, NK), pk[0], np.float32)
    f[15:NX - 15, 15:NX - 15, :] = pk[None, None, :]
    return f.ravel(order="F")


def _run(eps_r=1.0, mu_r=1.0, sigma=0.0, sigma_m=0.0):
    o = oracle.OracleSim("f64")
    o.set_params(pml=PML, tfsf_width=W)
    o.set_const([1e9, DX, DT], [STEPS, NX, NX, NK, 2])
    # probes: the scattered-field region above the box (z = 69), and z = 58
    o.set_antenna_locations(np.asfortranarray(np.array([[56, 56, 61], [56, 56, 50]], np.int32)))
    for f, half in ((1, False), (2, False), (3, True)):
        o.update_material(f, _cells(_profile(sigma, half, 0.0)))
    for f, half in ((4, False), (5, False), (6, True)):
        o.update_material(f, _cells(_profile(eps_r, half)))
    o.ready_simulation()
    if mu_r != 1.0 or sigma_m:
        mu = [_cells(_profile(mu_r, h)) for h in (True, True, False)]
        sm = [_cells(_profile(sigma_m, h, 0.0)) for h in (True, True, False)]
        o.set_magnetic(mu, sm if sigma_m else None)
    tau = FDIV * DX / (math.pi * C0)
    t = np.arange(STEPS) * np.float32(DT)
    pw = (-(t - 4 * tau) / tau * np.exp(-((t - 4 * tau) / tau) ** 2)).astype(np.float32)
    o.init_1d(1.0, pw)
    o.update_cuda()
    o.reset_field_all()
    for n in range(STEPS):
        o.step(n, 1)
    return np.asarray(o.array("probes"), np.float64).reshape(STEPS, 2, 6)


@pytest.fixture(scope="module")
def runs():
    oracle.build()
    s = 0.1 * EPS0 / DT  # sigma dt / (2 eps0) = 0.05
    return {"vac": _run(), "eps": _run(eps_r=4.0), "mu": _run(mu_r=4.0),
            "matched": _run(eps_r=4.0, mu_r=4.0),
            "lossy": _run(sigma=s, sigma_m=s * MU0 / EPS0)}


def _reflection(runs, name, q):
    nf = 8192
    inc = np.zeros(nf)
    inc[:110] = runs["vac"][:110, 1, 1]  # Ey above the block, vacuum
    ref = np.zeros(nf)
    ref[40:125] = runs[name][40:125, 0, 1]  # Ey in the scattered-field region
    f = np.fft.rfftfreq(nf, DT)
    i = np.argmin(np.abs(f - q * C0 / (FDIV * DX)))
    return abs(np.fft.rfft(ref)[i]) / abs(np.fft.rfft(inc)[i])


@pytest.mark.parametrize("q", [0.1, 0.2, 0.3])
def test_eps_and_mu_steps_reflect_one_third(runs, q):
    for name in ("eps", "mu"):
        r = _reflection(runs, name, q)
        assert abs(r - 1 / 3) < 6e-3, (name, q, r)


def test_mu_block_reflects_the_negative_of_the_eps_block(runs):
    re, rm = runs["eps"][40:125, 0, 1], runs["mu"][40:125, 0, 1]
    assert np.abs(re).max() > 0.1 * np.abs(runs["vac"][:, 1, 1]).max()
    assert np.dot(re, rm) / (np.linalg.norm(re) * np.linalg.norm(rm)) < -0.99


@pytest.mark.parametrize("q", [0.1, 0.2, 0.3])
def test_impedance_matched_blocks_do_not_reflect(runs, q):
    assert _reflection(runs, "matched", q) < 0.012
    assert _reflection(runs, "lossy", q) < 0.01

