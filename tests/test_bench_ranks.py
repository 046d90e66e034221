"""bench.py under a 2-rank torch.distributed launch (gloo, CPU only).

Replicas only: every rank would run its own copy of the case; the reference
arm (the CPU oracle) runs on rank 0 alone and prints one JSON line while the
other rank exits cleanly.  The GPU arm's multi-rank timing (barriers around
the timed region, max over ranks, the whole-job value) runs through the same
helpers of bench.py in tests/rank_timing_worker.py.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "3", "--warmup", "3",
           "--case", "t2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_gpu_arm_rank_timing():
    """The GPU arm's multi-rank timing on two gloo ranks: barriers around the
    timed region, the slowest rank's time on every rank (all-reduce MAX), and
    the whole-job value world x units x steps / that time."""
    pytest.importorskip("torch")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "tests", "rank_timing_worker.py")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    out = [l for l in r.stdout.splitlines() if l.startswith("[")]
    assert len(out) == 1, r.stdout
    lines = json.loads(out[0])
    assert sorted(d["rank"] for d in lines) == [0, 1]
    for d in lines:
        assert d["world"] == 2 and d["t_max"] == 2.0
        assert d["value"] == 2 * 1000 * 10 / 2.0
