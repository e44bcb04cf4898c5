"""One rank of the two-rank CPU check of bench.py's multi-process path
(launched by tests/test_bench_dist.py through torch.distributed.run)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def main(out_dir: str):
    world, rank, local = bench.dist_setup()
    # each rank's "step time" differs; every rank must see the maximum
    t = bench.dist_max(0.5 + rank, world)
    bench.dist_barrier(world)
    # the reference arm runs on rank 0 only: the other ranks return no line
    ref = None
    if rank != 0:
        ref = bench.run_reference_arm(None, dict(bench.WORKLOADS["life"], name="life"), world, rank)
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps(
        {"rank": rank, "local": local, "world": world, "max": t, "ref_line": ref}))
    bench.dist_barrier(world)


if __name__ == "__main__":
    main(sys.argv[1])
