"""The full-size workloads the benchmark times, run through the C ABI exactly
as the benchmark runs them and compared bit for bit with the reference's own
runIterativeCPU on the same seeded inputs.

The reference's results are too large to ship, so ``tests/golden/fullsize.json``
holds their SHA-256 (and the residual norms), written by
``tests/golden/make_fullsize.py`` from ``oracle/_ref/pskel_ref`` -- the
reference headers compiled unchanged apart from their CUDA-only members
(PSkelStencil.hpp:880-938 runIterativeCPU; the Life rule :389-440). The
inputs are regenerated here from their seeds and checked against the
fingerprints' input hashes first, so a generator change cannot pass silently.
"""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import bench
import pskel_gb300 as P
from pskel_gb300 import synth as S
from tests.golden import make_fullsize as F

pytestmark = pytest.mark.gpu

FP = json.loads((Path(__file__).resolve().parent / "golden" / "fullsize.json").read_text())


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_life_headline_run_matches_reference(cuda):
    """Game of Life 8192^2, Bernoulli(0.3) seed 1, 1000 generations, with the
    benchmark's schedule, on device buffers and through the host entry point."""
    torch = cuda
    fp = FP["life"]
    a, b = F.life_inputs()
    assert sha(a, b) == fp["input_sha"]
    keep = P._Keep()
    st = P.make_stencil(P.OP_LIFE, "u8", S.MOORE8_OFFSETS, keep=keep)
    T = bench.WORKLOADS["life"]["T"]
    x = torch.from_numpy(a).cuda()
    y = torch.from_numpy(b).cuda()
    P.iterate2d(st, x, y, fp["iterations"], sched=P.Schedule(time_steps=T))
    P.sync()
    got = (y if fp["iterations"] % 2 else x).cpu().numpy()
    assert sha(got) == fp["result_sha"], "device run differs from the reference"
    out = b.copy()
    P.run2d_host(st, a, out, fp["iterations"], sched=P.Schedule(time_steps=T))
    assert sha(out) == fp["result_sha"], "host entry point differs from the reference"


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_heat3d_full_run_matches_reference(cuda, dtype):
    """3D 7-point heat 512^3, 50 iterations, FP64 residual norm every 10 steps,
    with the benchmark's schedule: the grid bit for bit; the five norms to
    1e-12 relative of the exactly summed norms of the same states, and to
    2e-8 of the reference's own norms: the reference adds the 134M squares
    left to right in fp64, whose rounding error bound is (N-1) 2^-53 = 1.5e-8
    relative on the sum (about 1e-10 in fact)."""
    torch = cuda
    name = "heat3d" if dtype == "f32" else "heat3d_bf16"
    fp = FP[name]
    a, b = F.heat3d_inputs(dtype)
    assert sha(a, b) == fp["input_sha"]
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, keep=keep)
    wl = bench.WORKLOADS[name]
    view = (lambda v: torch.from_numpy(v.view(np.int16))) if dtype == "bf16" else torch.from_numpy
    x, y = view(a).cuda(), view(b).cuda()
    iters, every = fp["iterations"], fp["every"]
    res = torch.zeros(iters // every, dtype=torch.float64, device="cuda")
    P.iterate3d(st, x, y, iters, sched=P.Schedule(time_steps=wl["T"]), residual_every=every, residuals=res)
    P.sync()
    got = (y if iters % 2 else x).cpu().numpy()
    if dtype == "bf16":
        got = got.view(np.uint16)
    assert sha(got) == fp["result_sha"], "grid differs from the reference"
    got_norms = res.cpu().numpy()
    exact = np.array([float.fromhex(v) for v in fp["norms_exact"]])
    np.testing.assert_allclose(got_norms, exact, rtol=1e-12, atol=0)
    ref = np.array([float.fromhex(v) for v in fp["norms"]])
    np.testing.assert_allclose(got_norms, ref, rtol=2e-8, atol=0)
    print("RESIDUAL-ERROR", name, "vs exact", np.max(np.abs(got_norms - exact) / exact),
          "reference vs exact", np.max(np.abs(ref - exact) / exact))


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_batch_all_grids_match_reference(cuda, dtype):
    """All 256 grids of the batched workload (the benchmark's seed-1 draw and
    pool layout), in one persistent launch, with two uniform schedules and the
    library default: every grid's result bit for bit."""
    torch = cuda
    fp = FP["batch" if dtype == "f32" else "batch_bf16"]
    shapes = S.batch_shapes(256, seed=1)
    assert [(g["W"], g["H"], g["iterations"]) for g in fp["grids"]] == [tuple(map(int, s)) for s in shapes]
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    dev = torch.device("cuda", 0)
    host, pool, pool0, views = bench.batch_pool(torch, dev, shapes, dtype, seed=1)
    for k, ((W, H, _), (xv, yv, _p)) in enumerate(zip(shapes, views)):
        a = xv[:, :W].cpu().numpy()
        b = yv[:, :W].cpu().numpy()
        if dtype == "bf16":
            a, b = a.view(np.uint16), b.view(np.uint16)
        assert sha(a, b) == fp["grids"][k]["input_sha"], f"grid {k}: inputs differ"
    for T in (0, 5, 11):
        pool.copy_(pool0)
        batch = P.Batch(st, [(xv, yv, it, T, p, W) for (W, H, it), (xv, yv, p) in zip(shapes, views)])
        batch.run()
        P.sync()
        for k, ((W, H, it), (xv, yv, _p)) in enumerate(zip(shapes, views)):
            r = (yv if it % 2 else xv)[:, :W].cpu().numpy()
            if dtype == "bf16":
                r = r.view(np.uint16)
            assert sha(r) == fp["grids"][k]["result_sha"], f"T={T} grid {k} ({W}x{H}, {it} it) differs"
        batch.close()
