"""Game of Life on the GPU against the oracle: bit-exact (uint8 cells)."""
from __future__ import annotations

import numpy as np
import pytest

import pskel_gb300 as P
from pskel_gb300 import synth as S
from tests.gpu_util import run2d

pytestmark = pytest.mark.gpu


def life_stencil(keep, offsets=None, rng=0):
    return P.make_stencil(P.OP_LIFE, "u8", offsets or S.MOORE8_OFFSETS, rng=rng, keep=keep)


def grids(W, H, seed):
    a, _ = S.life(W, H, seed=seed)
    b = S.bernoulli_u8(seed + 1000, S.S_GRID, a.shape, 0.5)  # distinct ring in the output array
    return a, b


@pytest.mark.parametrize("W,H", [(67, 45), (224, 33), (225, 300), (1000, 777), (16, 16), (3, 3), (2, 50)])
@pytest.mark.parametrize("iters", [1, 2, 15, 17])
def test_life_matches_oracle(cuda, oracle_mod, W, H, iters):
    keep = P._Keep()
    a, b = grids(W, H, seed=W * 7 + H)
    got = run2d(cuda, life_stencil(keep), a, b, iters, dtype="u8")
    want = oracle_mod.life(a, b, iters)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("T", [1, 2, 3, 8, 13, 16, 21, 31])
@pytest.mark.parametrize("tile_h", [0, 2, 40])
def test_life_schedules(cuda, oracle_mod, T, tile_h):
    keep = P._Keep()
    a, b = grids(531, 407, seed=T)
    want = oracle_mod.life(a, b, 37)
    got = run2d(cuda, life_stencil(keep), a, b, 37, sched=dict(time_steps=T, tile_h=tile_h, ctas=0, tile_w=0, tile_d=0),
                dtype="u8")
    assert np.array_equal(got, want)


def test_life_mask_order_and_range(cuda, oracle_mod):
    keep = P._Keep()
    off = list(reversed(S.MOORE8_OFFSETS))
    a, b = grids(300, 200, seed=9)
    got = run2d(cuda, life_stencil(keep, off, rng=3), a, b, 9, dtype="u8")  # explicit range 3: ring of 3
    want = oracle_mod.life(a, b, 9, offsets=off, rng=3)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("pitch", [517, 520, 1024])
def test_life_pitched_and_unaligned(cuda, oracle_mod, pitch):
    # pitch 517 is not a multiple of 16 bytes: rows are packed with byte loads
    keep = P._Keep()
    a, b = grids(513, 301, seed=pitch)
    got = run2d(cuda, life_stencil(keep), a, b, 21, pitch=pitch, dtype="u8")
    assert np.array_equal(got, oracle_mod.life(a, b, 21))


def test_life_host_entry_point(cuda, oracle_mod):
    keep = P._Keep()
    for iters in (0, 1, 6, 33):
        a, b = grids(700, 513, seed=iters)
        a0 = a.copy()
        out = b.copy()
        P.run2d_host(life_stencil(keep), a, out, iters)
        assert np.array_equal(out, oracle_mod.life(a0, b, iters))
        assert np.array_equal(a, a0), "host input must not be modified"


def test_life_rejects_non_binary_cells(cuda):
    keep = P._Keep()
    a, b = grids(100, 100, seed=1)
    a[50, 50] = 2
    with pytest.raises(P.PskelError) as ei:
        run2d(cuda, life_stencil(keep), a, b, 3, dtype="u8")
    assert ei.value.status == P.PSKEL_ERR_DEVICE
    # the error is cleared; the next run succeeds
    a[50, 50] = 1
    run2d(cuda, life_stencil(keep), a, b, 3, dtype="u8")


def test_life_glider_known_answer_full_size(cuda):
    # A glider moves one cell down-right every 4 generations: after 4k steps the
    # grid is the initial one shifted by (k, k). 8192^2, 1000 generations.
    keep = P._Keep()
    N, gens = 8192, 1000
    a = np.zeros((N, N), dtype=np.uint8)
    g = np.array([[0, 1, 0], [0, 0, 1], [1, 1, 1]], dtype=np.uint8)
    a[10:13, 10:13] = g
    got = run2d(cuda, life_stencil(keep), a, a.copy(), gens, dtype="u8")
    want = np.zeros_like(a)
    k = gens // 4
    want[10 + k:13 + k, 10 + k:13 + k] = g
    assert np.array_equal(got, want)


def test_life_full_size_vs_oracle_and_schedule_invariance(cuda, oracle_mod):
    # 8192^2 Bernoulli(0.3): 24 generations against the oracle, and the full
    # 1000-generation run identical under two different temporal blockings.
    keep = P._Keep()
    a, b = S.life(8192, 8192, seed=1)
    got = run2d(cuda, life_stencil(keep), a, b, 24, dtype="u8")
    assert np.array_equal(got, oracle_mod.life(a, b, 24))
    r16 = run2d(cuda, life_stencil(keep), a, b, 1000, sched=dict(time_steps=16, tile_w=0, tile_h=0, tile_d=0, ctas=0),
                dtype="u8")
    r7 = run2d(cuda, life_stencil(keep), a, b, 1000, sched=dict(time_steps=7, tile_w=0, tile_h=100, tile_d=0, ctas=97),
               dtype="u8")
    assert np.array_equal(r16, r7)
    assert 0 < int(r16.sum()) < r16.size


@pytest.mark.parametrize("ctas", [1, 3])
def test_life_few_ctas_many_tiles(cuda, oracle_mod, ctas):
    # persistent CTAs walk many tiles each, ring tiles and interior ones
    keep = P._Keep()
    a, b = grids(1100, 600, seed=ctas)
    got = run2d(cuda, life_stencil(keep), a, b, 23,
                sched=dict(time_steps=9, tile_w=0, tile_h=50, tile_d=0, ctas=ctas), dtype="u8")
    assert np.array_equal(got, oracle_mod.life(a, b, 23))


@pytest.mark.parametrize("W,H", [(300, 1700), (333, 2100), (1000, 2500)])
@pytest.mark.parametrize("iters", [2, 3, 25, 26, 51, 200])
def test_life_host_run_overlapped(cuda, oracle_mod, W, H, iters):
    """pskel_run2d_host on grids of 8+ tile rows: rows are copied in and packed
    while the first passes run on the rows already there, and final rows are
    unpacked and copied out while the last passes run on the others."""
    keep = P._Keep()
    a, b = grids(W, H, seed=W + iters)
    got = P.run2d_host(life_stencil(keep), a, b.copy(), iters)
    assert np.array_equal(got, oracle_mod.life(a, b, iters))


@pytest.mark.parametrize("iters", [7, 60])
def test_life_host_run_overlapped_ring2(cuda, oracle_mod, iters):
    keep = P._Keep()
    a, b = grids(517, 1900, seed=iters)
    got = P.run2d_host(life_stencil(keep, rng=2), a, b.copy(), iters)
    assert np.array_equal(got, oracle_mod.life(a, b, iters, rng=2))
