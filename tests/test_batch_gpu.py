"""Batched 2D stencils (one persistent launch in a CUDA graph) against the
oracle, grid by grid, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import pskel_gb300 as P
from pskel_gb300 import synth as S
from tests.gpu_util import aligned_pitch, bits, from_dev, np_view, to_dev

pytestmark = pytest.mark.gpu


def make_grids(torch, n, seed, dtype, smin, smax, imax):
    rng = np.random.default_rng(seed)
    esz = 2 if dtype == "bf16" else 4
    out = []
    for i in range(n):
        W = int(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        H = int(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        it = int(rng.integers(1, imax + 1))
        T = int(rng.choice([0, 1, 3, 5, 7]))
        a, b = S.jacobi2d(W, H, seed=seed * 1000 + i)
        b = b.copy()
        b[0, :] = 0.5
        if dtype == "bf16":
            a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
        pitch = aligned_pitch(W, esz)
        x = to_dev(torch, np_view(a, dtype), pitch)
        y = to_dev(torch, np_view(b, dtype), pitch)
        out.append(dict(a=a, b=b, W=W, H=H, it=it, T=T, pitch=pitch, x=x, y=y, x0=x.clone(), y0=y.clone()))
    return out


def result(g, dtype):
    t = g["y"] if g["it"] % 2 == 1 else g["x"]
    r = from_dev(t, g["W"])
    return r.view(np.uint16) if dtype == "bf16" else r


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_batch_matches_oracle_per_grid(cuda, oracle_mod, dtype):
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    grids = make_grids(torch, 24, 5 if dtype == "f32" else 6, dtype, 16, 400, 40)
    batch = P.Batch(st, [(g["x"], g["y"], g["it"], g["T"], g["pitch"], g["W"]) for g in grids])
    assert batch.cell_updates == sum(g["W"] * g["H"] * g["it"] for g in grids)
    batch.run()
    P.sync()
    first = [result(g, dtype) for g in grids]
    for g, got in zip(grids, first):
        want = oracle_mod.lin2d(g["a"], g["b"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, g["it"], dtype=dtype)
        assert np.array_equal(bits(got), bits(want)), (g["W"], g["H"], g["it"], g["T"])
    # replay the graph from the same inputs: identical results
    for g in grids:
        g["x"].copy_(g["x0"])
        g["y"].copy_(g["y0"])
    batch.run()
    P.sync()
    for g, prev in zip(grids, first):
        assert np.array_equal(bits(result(g, dtype)), bits(prev))
    batch.close()


def test_batch_c5_like_distribution(cuda, oracle_mod):
    # side lengths log-uniform in [64, 512], iterations up to 60: many rounds,
    # grids finishing at different times, every grid checked
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    grids = make_grids(torch, 40, 11, "f32", 64, 512, 60)
    batch = P.Batch(st, [(g["x"], g["y"], g["it"], g["T"], g["pitch"], g["W"]) for g in grids])
    batch.run()
    P.sync()
    for g in grids:
        want = oracle_mod.lin2d(g["a"], g["b"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, g["it"])
        assert np.array_equal(bits(result(g, "f32")), bits(want))
    batch.close()


def test_batch_rejects_unsupported(cuda):
    torch = cuda
    keep = P._Keep()
    x = torch.zeros((64, 64), device="cuda")
    y = torch.zeros_like(x)
    st = P.make_stencil(P.OP_LINEAR, "f32", [(0, 0), (-2, 0)], [0.5, 0.5], keep=keep)
    with pytest.raises(P.PskelError) as ei:
        P.Batch(st, [(x, y, 3, 0)])
    assert ei.value.status == P.PSKEL_ERR_UNSUPPORTED


def c5_shapes(n=256, seed=2025, smin=64, smax=2048, imin=10, imax=500):
    """(W, H, iterations) of the batched workload's distribution: sides
    log-uniform in [smin, smax], iterations uniform in [imin, imax]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        W = int(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        H = int(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        out.append((W, H, int(rng.integers(imin, imax + 1))))
    return out


def test_batch_full_distribution(cuda, oracle_mod):
    """256 grids of the batched workload's distribution (670 MB of grids, more
    than L2) in one launch, 7 steps per pass: the cell-update count, a replay
    from the same inputs giving identical results, and the smallest grids
    against the oracle."""
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    grids = []
    for i, (W, H, it) in enumerate(c5_shapes()):
        pitch = aligned_pitch(W, 4)
        a = S.uniform_f32(7, i, (H, W))
        b = np.zeros_like(a)
        x = to_dev(torch, a, pitch)
        y = to_dev(torch, b, pitch)
        grids.append(dict(a=a, b=b, W=W, H=H, it=it, pitch=pitch, x=x, y=y, x0=x.clone()))
    batch = P.Batch(st, [(g["x"], g["y"], g["it"], 7, g["pitch"], g["W"]) for g in grids])
    assert batch.cell_updates == sum(g["W"] * g["H"] * g["it"] for g in grids)
    batch.run()
    P.sync()
    first = [result(g, "f32") for g in grids]
    for g in grids:
        g["x"].copy_(g["x0"])
        g["y"].zero_()
    batch.run()
    P.sync()
    assert all(np.array_equal(bits(result(g, "f32")), bits(f)) for g, f in zip(grids, first))
    for g, got in sorted(zip(grids, first), key=lambda t: t[0]["W"] * t[0]["H"] * t[0]["it"])[:8]:
        want = oracle_mod.lin2d(g["a"], g["b"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, g["it"])
        assert np.array_equal(bits(got), bits(want)), (g["W"], g["H"], g["it"])
    batch.close()
