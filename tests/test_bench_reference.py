"""bench.py's reference arm on CPU: the JSON line it prints for a workload
whose whole run fits one step (Jacobi 1024^2, 100 iterations)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "jacobi", "--steps", "2",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "GCells/s" and line["unit"] == "GCells/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 1
    # the same workload as the GPU arm, whole: 1024 x 1024, 100 iterations per step
    assert line["config"]["grid"] == [1024, 1024] and line["config"]["iterations_per_step"] == 100
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "whole workload" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "GCells/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the reference's own GPU path beside it: measured on a GPU node, marked unavailable here
    gp = line["gpu_path"]
    assert ("unavailable" in gp) if not Path("/dev/nvidiactl").exists() else gp["value"] > 0


def test_reference_arm_maps_no_library_of_ours():
    """The reference arm times only the reference: its process must not map
    libpskel_gb300.so (the seeded generators import without opening it)."""
    code = (
        "import argparse, bench\n"
        "a = argparse.Namespace(steps=1, warmup=1)\n"
        "line = bench.run_reference_arm(a, dict(bench.WORKLOADS['jacobi'], name='jacobi'), 1, 0)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPPED' if 'libpskel_gb300' in maps else 'CLEAN', line['value'] > 0)\n"
    )
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.split() == ["CLEAN", "True"], r.stdout
