"""Fingerprints of the reference's results on the full-size workloads.

Runs the reference's own ``runIterativeCPU`` (``oracle/_ref/pskel_ref``, built
from the reference headers by ``oracle/make_ref.py``) on the full-size seeded
workloads the benchmark times, and stores the SHA-256 of each result array --
and the residual norms as hexadecimal floats, both as the reference sums them
and summed exactly over the same states -- in ``tests/golden/fullsize.json``. The GPU tests run the same workloads through
the library's C ABI and compare bit for bit against these fingerprints, so the
full runs are pinned to the reference itself without shipping the arrays:

* Game of Life 8192 x 8192, Bernoulli(0.3) seed 1, 1000 generations;
* 3D 7-point heat 512^3, seed 1, 50 iterations, residual norm every 10 steps,
  fp32 and bf16 storage;
* the 256 grids of the batched Jacobi workload (seed 1), fp32 and bf16.

The inputs are regenerated by ``pskel_gb300.synth`` (their own SHA-256 is
stored too, so a generator change is caught). About 10 minutes on 8 cores.

    python tests/golden/make_fullsize.py [life heat3d heat3d_bf16 batch batch_bf16]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from pskel_gb300 import synth as S  # noqa: E402

OUT = Path(__file__).resolve().parent / "fullsize.json"
THREADS = os.cpu_count() or 1


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def life_inputs():
    return S.life(8192, 8192, seed=1)


def heat3d_inputs(dtype):
    a, b = S.heat3d(512, 512, 512, seed=1)
    if dtype == "bf16":
        a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
    return a, b


def batch_inputs(dtype, k, W, H):
    """Grid k of the batched workload (the benchmark's seed-1 draw)."""
    a, b = S.jacobi2d(W, H, seed=1 * 100003 + k)
    if dtype == "bf16":
        a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
    return a, b


def make_life():
    a, b = life_inputs()
    t = time.time()
    res, _ = oracle.ref_life(a, b, 1000, threads=THREADS)
    return {"input_sha": sha(a, b), "iterations": 1000, "result_sha": sha(res), "ref_s": round(time.time() - t, 1)}


def exact_norms(a, b, dtype, iters, every):
    """||u_k - u_{k-1}||_2 at k = every, 2 every, ..., summed exactly
    (math.fsum, then one rounding) over the states of the oracle's C
    restatement, which the golden fixtures pin bit for bit to the reference.
    The reference itself sums the squares left to right in fp64, whose
    rounding error on 134M terms reaches ~1e-10 relative."""
    import math
    x = a
    out = []
    for k in range(1, iters + 1):
        y, _ = oracle.lin3d(x, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 1, halo=0.0, dtype=dtype)
        if k % every == 0:
            xf = S.bf16_to_f32(x) if dtype == "bf16" else x
            yf = S.bf16_to_f32(y) if dtype == "bf16" else y
            d = yf.astype(np.float64).ravel() - xf.astype(np.float64).ravel()
            out.append(math.sqrt(math.fsum(d * d)))
        x = y
    return out, x


def make_heat3d(dtype):
    a, b = heat3d_inputs(dtype)
    t = time.time()
    res, norms = oracle.ref_lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 50, halo=0.0, dtype=dtype, every=10,
                                  threads=THREADS)
    ref_s = round(time.time() - t, 1)
    exact, last = exact_norms(a, b, dtype, 50, 10)
    assert sha(last) == sha(res), "the oracle's states differ from the reference's"
    return {"input_sha": sha(a, b), "iterations": 50, "every": 10, "result_sha": sha(res),
            "norms": [float(x).hex() for x in norms], "norms_exact": [float(x).hex() for x in exact],
            "ref_s": ref_s}


def make_batch(dtype):
    shapes = S.batch_shapes(256, seed=1)
    grids = []
    t = time.time()
    for k, (W, H, it) in enumerate(shapes):
        a, b = batch_inputs(dtype, k, W, H)
        res = oracle.ref_lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, it, dtype=dtype, threads=THREADS)
        grids.append({"W": int(W), "H": int(H), "iterations": int(it), "input_sha": sha(a, b),
                      "result_sha": sha(res)})
    return {"grids": grids, "ref_s": round(time.time() - t, 1)}


MAKERS = {"life": make_life, "heat3d": lambda: make_heat3d("f32"), "heat3d_bf16": lambda: make_heat3d("bf16"),
          "batch": lambda: make_batch("f32"), "batch_bf16": lambda: make_batch("bf16")}


def main(names):
    if not oracle.have_ref():
        oracle.build_ref()
    if not oracle.have_ref():
        raise SystemExit("oracle/_ref/pskel_ref is not built (needs the reference headers)")
    store = json.loads(OUT.read_text()) if OUT.exists() else {}
    for name in names:
        store[name] = MAKERS[name]()
        OUT.write_text(json.dumps(store, indent=1) + "\n")
        print(f"{name}: {store[name].get('ref_s')} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(MAKERS))
