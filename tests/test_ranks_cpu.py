"""The multi-process host path of bench.py (replicas, one process per GPU):
two gloo ranks on CPU agree on the barrier and on the maximum over ranks
that the whole-job timing takes, and a rank that raises surfaces as a
failed child process rather than a hang."""
import os
import socket
import subprocess
import sys
import textwrap

import pytest

from conftest import ROOT

CHILD = textwrap.dedent("""
    import os, sys
    sys.path.insert(0, {root!r})
    import bench
    r = bench.Ranks()
    r.barrier()
    v = r.max(float(10 + r.rank))
    r.barrier()
    print("RANK", r.rank, "WORLD", r.world, "MAX", v, flush=True)
    if os.environ.get("FAIL_RANK") == str(r.rank):
        raise SystemExit(3)
    r.close()
""")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(world, extra_env=None, timeout=120):
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=timeout) for p in procs]
    return procs, outs


def test_two_gloo_ranks_take_the_max():
    pytest.importorskip("torch")
    procs, outs = _launch(2)
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    lines = sorted(o.strip().splitlines()[-1] for o, _ in outs)
    assert lines == ["RANK 0 WORLD 2 MAX 11.0", "RANK 1 WORLD 2 MAX 11.0"]


def test_failing_rank_is_reported():
    pytest.importorskip("torch")
    procs, outs = _launch(2, {"FAIL_RANK": "1"})
    assert procs[1].returncode == 3
    assert procs[0].returncode == 0
