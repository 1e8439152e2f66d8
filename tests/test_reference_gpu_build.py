"""The reference's kernels build for sm_103a (no GPU needed): the recipe
compiles src/gpu.h through NVRTC and records every kernel the GPU parity
tests launch."""
import json
import os

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_kernels_build():
    ref = os.environ.get("MAXWELL_REF") or os.path.join(os.path.dirname(ROOT), "reference")
    if oracle.reference_root(ref) is None:
        pytest.skip("reference sources absent")
    out = oracle.build_reference_gpu(ref)
    from oracle.ref_gpu_build import KERNELS

    with open(os.path.join(out, "ref_gpu_names.json")) as f:
        meta = json.load(f)
    assert meta["arch"] == "sm_103a"
    assert sorted(meta["kernels"]) == sorted(KERNELS)
    for name in ("ref_gpu.cubin", "ref_gpu_nofma.cubin"):
        assert os.path.getsize(os.path.join(out, name)) > 0
