"""The register-resident Life tile, modelled on the CPU word for word.

life_bits_persistent_kernel (pskel_gb300/csrc/life.cu) advances a tile of
the bit plane T steps per pass with the tile in registers: a warp spans 32
words (lane l holds word 30*tx - 1 + l; lanes 1..30 are the core), warp w of
a block holds rows w*R .. w*R + R + 1 of the tile's window, a step computes
each warp's rows 1..R with west/east words from the adjacent lanes (a lane
without a neighbour gets its own word, as a warp shuffle does), and the warps
then exchange their first and last rows; tiles that reach the ring keep the
interior mask M and the ring flip D = src ^ dst outside M and write
M ? rule : old ^ D. This test restates exactly that on uint32 words, runs
whole multi-pass runs tile by tile, and compares with the oracle's
step-by-step run (the reference's ring semantics, PSkelStencil.hpp:2197-2257)
for odd sizes, rings of width 1 and 2 that differ between the two buffers,
partial tiles and several steps per pass. A core one row taller than the
window allows, or an exchange skipped, is caught by the same check.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from pskel_gb300 import synth as S

CORE = 30  # core words per tile (kernels.h)
# (consumer warps per block, rows per lane): the kernel's two geometries
# (kernels.h: 24 rows for passes of 15 steps or more, 16 for shorter ones)
# first; a window a third as tall checks the same scheme with more tiles
VARIANTS = [(15, 24), (15, 16), (15, 8)]


def words(W):
    return ((W + 31) // 32 + 3) & ~3


def pack(a):
    H, W = a.shape
    PW = words(W)
    bits = np.zeros((H, PW * 32), dtype=np.uint64)
    bits[:, :W] = a & 1
    wts = (np.uint64(1) << np.arange(32, dtype=np.uint64))
    return (bits.reshape(H, PW, 32) * wts).sum(axis=2).astype(np.uint32)


def unpack(p, W):
    H, PW = p.shape
    b = (p[:, :, None] >> np.arange(32, dtype=np.uint32)) & np.uint32(1)
    return b.reshape(H, PW * 32)[:, :W].astype(np.uint8)


def maj(a, b, c):
    return (a & b) | (a & c) | (b & c)


def row_sums(c):
    l = np.concatenate([c[..., :1], c[..., :-1]], axis=-1)  # shfl.up: lane 0 keeps its own word
    e = np.concatenate([c[..., 1:], c[..., -1:]], axis=-1)  # shfl.down: lane 31 keeps its own word
    we = (c << np.uint32(1)) | (l >> np.uint32(31))
    ea = (c >> np.uint32(1)) | (e << np.uint32(31))
    return we ^ c ^ ea, maj(we, c, ea), we ^ ea, we & ea


def step(x, ring_md):
    """x: (warps, R+2, 32) words; rows 1..R of every warp advance one step."""
    t0, t1, p0, p1 = row_sums(x)
    s0 = t0[:, :-2] ^ p0[:, 1:-1] ^ t0[:, 2:]
    k0 = maj(t0[:, :-2], p0[:, 1:-1], t0[:, 2:])
    x1 = t1[:, :-2] ^ p1[:, 1:-1] ^ t1[:, 2:]
    y1 = maj(t1[:, :-2], p1[:, 1:-1], t1[:, 2:])
    c = x[:, 1:-1]
    alive = (~y1 & (x1 ^ k0)) & (s0 | c)
    if ring_md is not None:
        m, d = ring_md
        alive = (m & alive) | (~m & (c ^ d))
    x[:, 1:-1] = alive


def bit_range(lo, hi):
    lo, hi = max(0, min(32, lo)), max(0, min(32, hi))
    if hi <= lo:
        return np.uint32(0)
    return np.uint32(((1 << hi) - 1) & ~((1 << lo) - 1))


def run_tile(src, dst, out, W, H, ring, T, TH, steps, ty, tx, NW, R, exchange=True, extra_core=0):
    PW = src.shape[1]
    WINDOW = NW * R + 2
    wy0 = ty * TH - T
    lanes = np.arange(32)
    gw = tx * CORE - 1 + lanes
    gw_in = (gw >= 0) & (gw < PW)
    rows = wy0 + np.arange(NW)[:, None] * R + np.arange(R + 2)[None, :]  # (NW, R+2)
    inside = (rows >= 0) & (rows < H)

    def load(plane):
        v = np.zeros((NW, R + 2, 32), dtype=np.uint32)
        ok = inside[:, :, None] & gw_in[None, None, :]
        rr = np.clip(rows, 0, H - 1)[:, :, None].repeat(32, axis=2)
        cc = np.clip(gw, 0, PW - 1)[None, None, :].repeat(NW, axis=0).repeat(R + 2, axis=1)
        v[ok] = plane[rr[ok], cc[ok]]
        return v

    x = load(src)
    ring_tile = (wy0 < ring or wy0 + WINDOW > H - ring or (tx * CORE - 1) * 32 < ring
                 or (tx * CORE + 31) * 32 > W - ring)
    md = None
    if ring_tile:
        b = load(dst)[:, 1:-1]
        colmask = np.array([bit_range(ring - 32 * g, (W - ring) - 32 * g) if ok else 0
                            for g, ok in zip(gw, gw_in)], dtype=np.uint32)
        r_in = (rows[:, 1:-1] >= ring) & (rows[:, 1:-1] < H - ring) & inside[:, 1:-1]
        m = np.where(r_in[:, :, None], colmask[None, None, :], np.uint32(0)).astype(np.uint32)
        md = (m, (x[:, 1:-1] ^ b) & ~m)
    for s in range(steps):
        step(x, md)
        if s + 1 < steps and exchange:
            first, last = x[:, 1].copy(), x[:, R].copy()
            x[1:, 0] = last[:-1]
            x[:-1, R + 1] = first[1:]
    gc0, gc1 = ty * TH - extra_core, min(H, ty * TH + TH + extra_core)
    for w in range(NW):
        for i in range(1, R + 1):
            gy = rows[w, i]
            if gc0 <= gy < gc1 and 0 <= gy < H:
                for l in range(1, CORE + 1):
                    if gw[l] < PW:
                        out[gy, gw[l]] = x[w, i, l]


def plan_passes(iters, T):
    p = [T] * (iters // T) + ([iters % T] if iters % T else [])
    if len(p) % 2 != iters % 2:
        for i, v in enumerate(p):
            if v >= 2:
                p[i:i + 1] = [v // 2, v - v // 2]
                break
    return p


def model_life(a, b, iters, T, ring=1, TH=None, variant=VARIANTS[0], **kw):
    """The kernel's run on two bit planes; returns the result array (the
    interior of the final plane over the result buffer's own ring)."""
    H, W = a.shape
    NW, R = variant
    TH = TH or NW * R + 2 - 2 * T
    X, Y = pack(a), pack(b)
    PW = X.shape[1]
    tiles_x, tiles_y = math.ceil(PW / CORE), math.ceil(H / TH)
    passes = plan_passes(iters, T)
    for i, steps in enumerate(passes):
        src, dst = (X, Y) if i % 2 == 0 else (Y, X)
        out = dst.copy()
        for ty in range(tiles_y):
            for tx in range(tiles_x):
                run_tile(src, dst, out, W, H, ring, T, TH, steps, ty, tx, NW, R, **kw)
        if i % 2 == 0:
            Y = out
        else:
            X = out
    fin = Y if len(passes) % 2 else X
    res = (b if len(passes) % 2 else a).copy()
    inner = unpack(fin, W)
    res[ring:H - ring, ring:W - ring] = inner[ring:H - ring, ring:W - ring]
    return res


def grids(W, H, seed):
    a, _ = S.life(W, H, seed=seed)
    b = S.bernoulli_u8(seed + 1000, S.S_GRID, a.shape, 0.5)  # a ring of its own in the output array
    return a, b


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("W,H,iters,T", [(67, 45, 9, 3), (1000, 300, 13, 13), (2000, 520, 17, 7),
                                         (961, 123, 5, 5), (33, 129, 4, 1), (1024, 260, 31, 31)])
def test_tile_model_matches_oracle(oracle_mod, W, H, iters, T, variant):
    a, b = grids(W, H, seed=W + H)
    want = oracle_mod.life(a, b, iters)
    if variant[0] * variant[1] + 2 - 2 * T < 1:
        pytest.skip("no tile height fits")
    assert np.array_equal(model_life(a, b, iters, T, variant=variant), want)


def test_tile_model_wide_ring(oracle_mod):
    a, b = grids(700, 400, seed=5)
    want = oracle_mod.life(a, b, 11, rng=2)
    assert np.array_equal(model_life(a, b, 11, 5, ring=2), want)


def test_tile_model_shorter_tiles(oracle_mod):
    a, b = grids(900, 333, seed=6)
    want = oracle_mod.life(a, b, 15)
    assert np.array_equal(model_life(a, b, 15, 7, TH=40), want)


def test_planted_mistakes_are_caught(oracle_mod):
    # taller than one core, so that a core boundary falls inside the grid
    a, b = grids(1000, 700, seed=7)
    want = oracle_mod.life(a, b, 13)
    assert not np.array_equal(model_life(a, b, 13, 13, exchange=False), want)
    assert not np.array_equal(model_life(a, b, 13, 13, extra_core=1), want)
