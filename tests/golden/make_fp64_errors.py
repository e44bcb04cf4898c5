"""Errors of the benchmark's floating-point workloads against an FP64 oracle.

Every float result of the library is bit-identical to the oracle's fp32 / bf16
restatement on the same inputs (the ``-m gpu`` suite checks the full-size runs:
``tests/test_fullsize_gpu.py``, ``test_advection_c3_full_size_and_fp64_error``
and the Jacobi 1024^2 test in ``tests/test_stencil2d_gpu.py``). So the error of
a benchmark run against FP64 is the error of that restatement against the same
algorithm evaluated in double precision on the same inputs (bf16 inputs and
winds widened exactly), which this script computes on the CPU and stores in
``tests/golden/fp64_errors.json``; ``bench.py`` reports it beside each float
workload. Per workload: the largest absolute error, the largest relative error
over cells whose FP64 value exceeds 1e-6 in magnitude, and the relative L2
error ||x - x64|| / ||x64||, over the whole result grid (all 256 grids for the
batch).

    python tests/golden/make_fp64_errors.py [workload ...]
"""
from __future__ import annotations

import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
import oracle  # noqa: E402
from pskel_gb300 import synth as S  # noqa: E402

OUT = Path(__file__).resolve().parent / "fp64_errors.json"
FLOAT_WORKLOADS = ["jacobi", "jacobi_bf16", "advect", "advect_bf16", "heat3d", "heat3d_bf16", "batch", "batch_bf16"]


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def widen(x, dtype):
    return (S.bf16_to_f32(x) if dtype == "bf16" else x).astype(np.float64)


class Acc:
    """Error statistics accumulated over one or more result grids."""

    def __init__(self):
        self.max_abs = 0.0
        self.max_rel = 0.0
        self.d2 = 0.0
        self.r2 = 0.0

    def add(self, got, ref):
        d = np.abs(got - ref)
        self.max_abs = max(self.max_abs, float(d.max(initial=0.0)))
        big = np.abs(ref) > 1e-6
        if big.any():
            self.max_rel = max(self.max_rel, float((d[big] / np.abs(ref[big])).max()))
        self.d2 += float(np.sum(d * d))
        self.r2 += float(np.sum(ref * ref))

    def result(self):
        return {"max_abs": self.max_abs, "max_rel": self.max_rel,
                "rel_l2": (self.d2 ** 0.5) / (self.r2 ** 0.5) if self.r2 > 0 else 0.0}


def run_grid(name, dtype, x, iters):
    """(low-precision result widened, FP64 result) of one grid."""
    if name.startswith(("jacobi", "batch")):
        lo = oracle.lin2d(x["in"], x["out"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters, dtype=dtype)
        hi = oracle.lin2d(widen(x["in"], dtype), widen(x["out"], dtype), S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters,
                          dtype="f64")
    elif name.startswith("advect"):
        lo = oracle.advect(x["in"], x["out"], x["u"], x["v"], iters, S.ADVECT_K, S.ADVECT_DT, S.ADVECT_INV_DX,
                           dtype=dtype)
        hi = oracle.advect(widen(x["in"], dtype), widen(x["out"], dtype), widen(x["u"], dtype), widen(x["v"], dtype),
                           iters, S.ADVECT_K, S.ADVECT_DT, S.ADVECT_INV_DX, dtype="f64")
    else:
        lo, _ = oracle.lin3d(x["in"], x["out"], S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=0.0, dtype=dtype)
        hi, _ = oracle.lin3d(widen(x["in"], dtype), widen(x["out"], dtype), S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters,
                             halo=0.0, dtype="f64")
    return widen(lo, dtype), hi


def make(name):
    wl = dict(bench.WORKLOADS[name], name=name)
    dtype = wl["dtype"]
    acc = Acc()
    t = time.time()
    if wl.get("batch"):
        shapes = S.batch_shapes(256, seed=1)
        h = hashlib.sha256()
        for k, (W, H, it) in enumerate(shapes):
            a, b = S.jacobi2d(int(W), int(H), seed=1 * 100003 + k)
            if dtype == "bf16":
                a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
            h.update(a.tobytes())
            h.update(b.tobytes())
            lo, hi = run_grid(name, dtype, {"in": a, "out": b}, int(it))
            acc.add(lo, hi)
        input_sha = h.hexdigest()
        iters = "per grid (uniform [10, 500])"
    else:
        x = bench.make_inputs(wl)
        input_sha = sha(*x.values())
        iters = wl["iters"]
        lo, hi = run_grid(name, dtype, x, iters)
        acc.add(lo, hi)
    return dict(acc.result(), dtype=dtype, iterations=iters, input_sha=input_sha, cpu_s=round(time.time() - t, 1))


def main(names):
    oracle.build()
    store = json.loads(OUT.read_text()) if OUT.exists() else {}
    for name in names:
        store[name] = make(name)
        OUT.write_text(json.dumps(store, indent=1, sort_keys=True) + "\n")
        print(name, store[name], flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or FLOAT_WORKLOADS)
