"""Pins the CPU oracle to the reference: every scenario's outputs from the
oracle's FP32 build must equal the golden vectors produced by the
reference's own sources (tests/golden/make_golden.py) bit for bit, and the
FP64 build must agree with them to the FP32 rounding floor."""
import hashlib
import os

import numpy as np
import pytest

from scenarios import SCENARIOS, run_oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
COEFS = ("Cexe", "Ceye", "Ceze", "Cexh", "Ceyh", "Cezh")
PSI = ("Exy", "Ezy", "Hxy", "Hzy", "Exz", "Eyz", "Hxz", "Hyz", "Eyx", "Ezx", "Hyx", "Hzx")


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def _golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def _inputs_from_golden(g, sc):
    return dict(
        freqRes=g["in_freqRes"], TimeDim=g["in_TimeDim"], pw=g["in_pw"],
        source=g["in_source"], mats={f: g[f"in_mat{f}"] for f in range(1, 7)},
        probes=g.get("in_probes"))


@pytest.mark.parametrize("sc", SCENARIOS, ids=lambda s: s.name)
def test_oracle_bit_exact_vs_reference(sc):
    g = _golden(sc.name)
    o = run_oracle(sc, "f32", inp=_inputs_from_golden(g, sc))
    np.testing.assert_array_equal(o.array("b_E"), g["b_E"])
    np.testing.assert_array_equal(o.array("c_E"), g["c_E"])
    np.testing.assert_array_equal(o.array("b_H"), g["b_H"])
    np.testing.assert_array_equal(o.array("c_H"), g["c_H"])
    np.testing.assert_array_equal(o.array("den_ex"), g["den_ex"])
    np.testing.assert_array_equal(o.array("den_hx"), g["den_hx"])
    assert np.float32(o.scalar("Che")) == g["Che"]
    assert np.float32(o.scalar("Chh")) == g["Chh"]
    for name in COEFS + FIELDS:
        a = o.field(name)
        assert np.array_equal(a[g["smp_index"]], g[f"smp_{name}"]), name
        assert _sha(a) == str(g[f"sha_{name}"]), name
    for name in PSI:
        assert _sha(o.psi(name)) == str(g[f"sha_psi_{name}"]), name
    if sc.mode:
        for name in ("Ez_1D", "Hy_1D", "E_inv_1D", "H_inv_1D"):
            assert _sha(o.array(name)) == str(g[f"sha_{name}"]), name


@pytest.mark.parametrize("sc", SCENARIOS[:3], ids=lambda s: s.name)
def test_oracle_fp64_floor(sc):
    """The FP64 build stays within the FP32 rounding floor of the pinned
    FP32 result (rel-L2 well under the 1e-5 parity tolerance)."""
    g = _golden(sc.name)
    inp = _inputs_from_golden(g, sc)
    o32 = run_oracle(sc, "f32", inp=inp)
    o64 = run_oracle(sc, "f64", inp=inp)
    for group in (FIELDS[:3], FIELDS[3:]):
        # per component, relative to the norm of the whole E (or H) field:
        # components that carry only rounding noise (e.g. Ex in mode 3
        # vacuum) have no meaningful relative error of their own
        scale = np.sqrt(sum(np.linalg.norm(o64.field(n)) ** 2 for n in group))
        for name in group:
            a, b = o32.field(name).astype(np.float64), o64.field(name)
            rel = np.linalg.norm(a - b) / max(scale, 1e-300)
            assert rel < 1e-5, (name, rel)
