"""Out-of-core runs (grids in host memory streamed through the GPU in slabs)
against the oracle.

pskel_run2d_host_tiled / pskel_run3d_host_tiled replace the host tiling of
runIterativeTilingGPU (PSkelStencil.hpp:1663-1760 of the reference). Each case
forces several slabs per pass (small slab heights or a small device budget),
several passes (inner iteration counts below the iteration count) and slabs
smaller than their halo, and compares the result bit for bit with the oracle,
which runs the whole grid step by step.
"""
from __future__ import annotations

import numpy as np
import pytest

import pskel_gb300 as P
from pskel_gb300 import synth as S
from tests.golden.make_golden import STAR9_OFFSETS, STAR9_WEIGHTS
from tests.gpu_util import bits

pytestmark = pytest.mark.gpu


def jac(W, H, seed, dtype):
    a, b = S.jacobi2d(W, H, seed=seed)
    b = b.copy()
    b[0, :] = 0.5
    b[:, -1] = 0.25
    if dtype == "bf16":
        return S.f32_to_bf16(a), S.f32_to_bf16(b)
    return a, b


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("iters", [1, 2, 7, 16, 45])
@pytest.mark.parametrize("slab,inner", [(5, 3), (64, 15), (300, 7), (1, 1), (33, 8)])
def test_jacobi_tiled(cuda, oracle_mod, dtype, iters, slab, inner):
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    a, b = jac(301, 203, iters + slab, dtype)
    a0 = a.copy()
    want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters, dtype=dtype)
    got = P.run2d_host_tiled(st, a, b.copy(), iters, slab_rows=slab, inner=inner)
    assert np.array_equal(bits(got), bits(want))
    assert np.array_equal(a, a0)  # the input array is not modified


@pytest.mark.parametrize("offsets,weights,rng", [
    (STAR9_OFFSETS, STAR9_WEIGHTS, 0),     # reach 2, ring 2
    (S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, 3),  # reach 1, ring 3
])
@pytest.mark.parametrize("iters", [3, 20])
def test_ring_wider_than_one(cuda, oracle_mod, offsets, weights, rng, iters):
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", offsets, weights, rng=rng, keep=keep)
    a = S.uniform_f32(3, 1, (157, 130))
    b = S.uniform_f32(3, 2, (157, 130))
    want = oracle_mod.lin2d(a, b, offsets, weights, iters, rng=rng)
    got = P.run2d_host_tiled(st, a, b.copy(), iters, slab_rows=9, inner=5)
    assert np.array_equal(bits(got), bits(want))


def test_device_budget_sizes_the_slabs(cuda, oracle_mod):
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    W, H, iters, inner = 1000, 2000, 27, 9  # passes 9, 9, 9
    budget = 6 << 20
    slab, halo, slabs, dev = P.tiled_plan(st, (H, W), iters, inner=inner, device_bytes=budget)
    assert slabs > 1 and dev <= budget and halo == 1 + (inner - 1)
    a, b = jac(W, H, 9, "f32")
    want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
    got = P.run2d_host_tiled(st, a, b.copy(), iters, inner=inner, device_bytes=budget)
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("iters", [1, 2, 17, 40])
@pytest.mark.parametrize("slab,inner", [(7, 5), (100, 15), (2, 1)])
def test_life_tiled(cuda, oracle_mod, iters, slab, inner):
    keep = P._Keep()
    st = P.make_stencil(P.OP_LIFE, "u8", S.MOORE8_OFFSETS, keep=keep)
    a, _ = S.life(345, 250, seed=iters)
    b = S.bernoulli_u8(iters + 1000, S.S_GRID, a.shape, 0.5)  # the output array's own ring
    want = oracle_mod.life(a, b, iters)
    got = P.run2d_host_tiled(st, a, b.copy(), iters, slab_rows=slab, inner=inner)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("iters,slab,inner", [(9, 11, 3), (16, 40, 7), (1, 8, 1)])
def test_advection_tiled(cuda, oracle_mod, dtype, iters, slab, inner):
    a, b, u, v = S.advect2d(190, 170, seed=iters)
    b = b.copy()
    b[-1, :] = 0.75
    if dtype == "bf16":
        a, b, u, v = (S.f32_to_bf16(x) for x in (a, b, u, v))
    u = np.ascontiguousarray(u)
    v = np.ascontiguousarray(v)
    keep = P._Keep()
    st = P.make_stencil(P.OP_ADVECT, dtype, S.JACOBI4_OFFSETS, wind=(u.ctypes.data, v.ctypes.data), K=S.ADVECT_K,
                        dt=S.ADVECT_DT, inv_dx=S.ADVECT_INV_DX, keep=keep)
    want = oracle_mod.advect(a, b, u, v, iters, S.ADVECT_K, S.ADVECT_DT, S.ADVECT_INV_DX, dtype=dtype)
    got = P.run2d_host_tiled(st, a, b.copy(), iters, slab_rows=slab, inner=inner)
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("iters,slab,inner", [(1, 4, 1), (2, 16, 3), (9, 5, 3), (14, 20, 15)])
def test_heat3d_tiled(cuda, oracle_mod, dtype, iters, slab, inner):
    a, _ = S.heat3d(40, 57, 72, seed=iters)
    b = S.uniform_f32(iters + 50, S.S_GRID, a.shape)
    if dtype == "bf16":
        a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, halo=0.5, keep=keep)
    want, _ = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=0.5, dtype=dtype)
    got = P.run3d_host_tiled(st, a, b.copy(), iters, slab_planes=slab, inner=inner)
    assert np.array_equal(bits(got), bits(want))


def test_zero_iterations_copies_the_input(cuda):
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    a, b = jac(50, 40, 1, "f32")
    got = P.run2d_host_tiled(st, a, b.copy(), 0, slab_rows=8)
    assert np.array_equal(got, a)


def test_same_as_in_core_host_run(cuda):
    """The out-of-core result equals pskel_run2d_host's on the same arrays."""
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    a, b = jac(2048, 1536, 4, "f32")
    ref = P.run2d_host(st, a, b.copy(), 60)
    got = P.run2d_host_tiled(st, a, b.copy(), 60, slab_rows=200, inner=15)
    assert np.array_equal(bits(got), bits(ref))
