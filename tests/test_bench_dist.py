"""bench.py under torchrun with two ranks, on CPU (gloo): the rendezvous on
127.0.0.1, the max-over-ranks step time every rank reports, the barrier, and
the reference arm running on rank 0 only."""
from __future__ import annotations

import json
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gloo(tmp_path):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "tests" / "dist_worker.py"), str(tmp_path)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    ranks = [json.loads((tmp_path / f"rank{i}.json").read_text()) for i in range(2)]
    assert [d["rank"] for d in ranks] == [0, 1]
    assert all(d["world"] == 2 for d in ranks)
    assert all(d["max"] == 1.5 for d in ranks)  # max over the ranks' 0.5 and 1.5
    assert ranks[1]["ref_line"] is None
