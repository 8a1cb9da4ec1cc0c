"""Multi-process replica logic of bench.py on the CPU: two gloo ranks each
cluster their copy of a small workload; rank 0 alone prints one JSON line
whose value is the summed work over the slowest rank's time."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_replicas_report_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", str(ROOT / "bench.py"), "--cpu-only",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--iters-per-step", "2", "--n-seqs", "120",
           "--workload", "dna_small"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["n_gpus"] == 2 and out["value"] > 0 and out["scaling"] == "weak"


def test_reference_arm_uses_oracle_code_only():
    """bench.py --impl reference times the oracle on the host cores with
    inputs built by oracle-side code: the product library is not mapped."""
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1",
           "--n-seqs", "3000", "--workload", "dna_small"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert out["impl"] == "reference" and out["value"] > 0
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["arch"]
    assert out["libraries"] and all(x.startswith("oracle/_build/") for x in out["libraries"]), out["libraries"]
