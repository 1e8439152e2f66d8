"""bench.py's reference arm runs on the host cores alone: one JSON line with
the metric, unit and config of our arm, at least three warm-up steps, and
the cpu_baseline / e2e objects the line must carry."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    pytest.importorskip("oracle")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "c1", "--steps", "2", "--warmup", "1"],
                         capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "Mcell-steps/s" and d["unit"] == "Mcell-steps/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["warmup"] >= 3 and d["steps"] >= 1 and d["value"] > 0
    assert d["config"]["workload"].startswith("c1:")
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0
