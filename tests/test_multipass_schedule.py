"""The one-launch 2D schedule, modelled on the CPU.

fast2d_multipass_kernel runs every pass of a run in one persistent launch:
items (pass i, tile t) are taken in order, and before staging its tile an
item waits until every tile of pass i-1 whose core overlaps its loaded tile
(ceil(HY/TH) tile rows and ceil(HX/TW) tile columns around it) has completed.
This test restates that schedule with loads and stores as separate events,
runs it under many random interleavings of the CTAs, and checks the result
against the step-by-step ping-pong of the reference (ring cells never
written, PSkelStencil.hpp:2197-2257). Each tile computes at step s only the
rows [s, LH - s) that are still exact, as the tile routine does. A wait set
one tile too small, or one row fewer computed, is caught by the same check.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

OFFS = [(-1, 0), (1, 0), (0, -1), (0, 1)]
WTS = [0.25, 0.25, 0.25, 0.25]


def step(src, dst, ring):
    """One step: interior cells of dst from src; dst's ring untouched."""
    H, W = src.shape
    out = dst.copy()
    acc = np.zeros((H - 2 * ring, W - 2 * ring))
    for (dh, dw), w in zip(OFFS, WTS):
        acc = acc + w * src[ring + dh:H - ring + dh, ring + dw:W - ring + dw]
    out[ring:H - ring, ring:W - ring] = acc
    return out


def reference(a, b, passes, ring):
    x, y = a.copy(), b.copy()
    for k in range(sum(passes)):
        if k % 2 == 0:
            y = step(x, y, ring)
        else:
            x = step(y, x, ring)
    return y if sum(passes) % 2 else x


def run_tile(bufs, i, t, steps, geo, ring, exact_margin=0):
    """Load phase of item (i, t): stage src (and dst for its ring) tiles,
    then the steps. Step s computes only the tile rows [s, LH - s), the rows
    still exact (exact_margin > 0 drops that many more on each side: a
    planted mistake); other rows keep whatever the buffer held."""
    H, W, TW, TH, HX, HY, tx_n = geo
    src, dst = (0, 1) if i % 2 == 0 else (1, 0)
    ty, tx = divmod(t, tx_n)
    gy0, gx0 = ty * TH - HY, tx * TW - HX
    LH, LW = TH + 2 * HY, TW + 2 * HX

    def stage(buf):
        tile = np.zeros((LH, LW))
        ys, xs = slice(max(gy0, 0), min(gy0 + LH, H)), slice(max(gx0, 0), min(gx0 + LW, W))
        tile[ys.start - gy0:ys.stop - gy0, xs.start - gx0:xs.stop - gx0] = bufs[buf][ys, xs]
        return tile

    s_tile, d_tile = stage(src), stage(dst)
    gy = np.arange(gy0, gy0 + LH)[:, None]
    gx = np.arange(gx0, gx0 + LW)[None, :]
    interior = (gy >= ring) & (gy < H - ring) & (gx >= ring) & (gx < W - ring)
    cur, other = s_tile, d_tile
    rows = np.arange(LH)[:, None]
    for s in range(1, steps + 1):
        nxt = other.copy()
        acc = np.zeros((LH - 2, LW - 2))
        for (dh, dw), w in zip(OFFS, WTS):
            acc = acc + w * cur[1 + dh:LH - 1 + dh, 1 + dw:LW - 1 + dw]
        live = (rows >= s + exact_margin) & (rows < LH - s - exact_margin)
        inner = (interior & live)[1:-1, 1:-1]
        nxt[1:-1, 1:-1][inner] = acc[inner]
        cur, other = nxt, cur
    # the store phase writes the core's interior cells into dst
    core = (slice(HY, HY + TH), slice(HX, HX + TW))
    return dst, gy0, gx0, cur[core], interior[core]


def store(bufs, dst, gy0, gx0, core, mask, geo):
    H, W, TW, TH, HX, HY, _ = geo
    y0, x0 = gy0 + HY, gx0 + HX
    ys, xs = slice(y0, min(y0 + TH, H)), slice(x0, min(x0 + TW, W))
    c = core[:ys.stop - y0, :xs.stop - x0]
    m = mask[:ys.stop - y0, :xs.stop - x0]
    region = bufs[dst][ys, xs]
    region[m] = c[m]


def simulate(a, b, passes, ring, TW, TH, T, ctas, rng, dy=None, dx=None, exact_margin=0):
    H, W = a.shape
    HY, HX = T, T
    tx_n, ty_n = math.ceil(W / TW), math.ceil(H / TH)
    ntiles = tx_n * ty_n
    geo = (H, W, TW, TH, HX, HY, tx_n)
    dy = math.ceil(HY / TH) if dy is None else dy
    dx = math.ceil(HX / TW) if dx is None else dx
    bufs = [a.copy(), b.copy()]
    done = np.zeros(ntiles, dtype=int)
    items = [(i, t) for i in range(len(passes)) for t in range(ntiles)]
    nxt = 0
    cta = [None] * ctas  # per CTA: None or [phase, item, staged]
    while nxt < len(items) or any(c is not None for c in cta):
        k = int(rng.integers(ctas))
        c = cta[k]
        if c is None:
            if nxt < len(items):
                cta[k] = ["wait", items[nxt], None]
                nxt += 1
            continue
        phase, (i, t), staged = c
        ty, tx = divmod(t, tx_n)
        if phase == "wait":
            ready = i == 0 or all(done[yy * tx_n + xx] >= i
                                  for yy in range(max(0, ty - dy), min(ty_n, ty + dy + 1))
                                  for xx in range(max(0, tx - dx), min(tx_n, tx + dx + 1)))
            if ready:
                c[0], c[2] = "stored", run_tile(bufs, i, t, passes[i], geo, ring, exact_margin)
        elif phase == "stored":
            store(bufs, *staged, geo)
            done[t] += 1
            cta[k] = None
    return bufs[1] if len(passes) % 2 else bufs[0]


# More CTAs than tiles per pass (as on the GPU: 304 CTAs for the 240 tiles
# of a 1024^2 Jacobi run) lets items of three passes be in flight at once.
@pytest.mark.parametrize("H,W,TW,TH,T,passes,ctas", [
    (37, 45, 8, 9, 3, [3, 3, 1], 5),
    (37, 45, 8, 9, 3, [3, 3, 1], 60),
    (40, 33, 6, 5, 5, [5, 3, 3, 1, 1], 7),
    (40, 33, 6, 5, 5, [5, 3, 3, 1, 1], 100),
    (29, 30, 12, 7, 7, [7, 5, 3], 3),
    (29, 30, 12, 7, 7, [7, 5, 3], 40),
    (24, 24, 4, 4, 3, [3, 3, 3, 1], 16),
    (24, 24, 4, 4, 3, [3, 3, 3, 1], 72),
    (30, 30, 8, 3, 5, [5, 5, 3], 90),  # halo taller than the core: waits reach two tile rows
])
def test_one_launch_schedule_matches_step_by_step(H, W, TW, TH, T, passes, ctas):
    rng = np.random.default_rng(H * W + T)
    a = rng.random((H, W))
    b = rng.random((H, W))
    want = reference(a, b, passes, 1)
    for trial in range(6):
        got = simulate(a, b, passes, 1, TW, TH, T, ctas, np.random.default_rng(trial))
        assert np.array_equal(got, want)


def test_a_smaller_wait_set_is_caught():
    # the same interleavings with the wait reaching no neighbouring tile row
    # give a wrong result: the check above is able to see a missing wait
    H, W, TW, TH, T, passes = 40, 33, 6, 5, 5, [5, 3, 3, 1, 1]
    rng = np.random.default_rng(3)
    a = rng.random((H, W))
    b = rng.random((H, W))
    want = reference(a, b, passes, 1)
    wrong = 0
    for trial in range(6):
        got = simulate(a, b, passes, 1, TW, TH, T, 100, np.random.default_rng(trial), dy=0)
        wrong += not np.array_equal(got, want)
    assert wrong > 0


def test_computing_one_row_fewer_is_caught():
    # the tile routine computes rows [s, LH - s) at step s; one row fewer on
    # each side leaves stale values inside the core after a full-length pass
    H, W, TW, TH, T, passes = 40, 33, 6, 5, 5, [5, 3, 3, 1, 1]
    rng = np.random.default_rng(4)
    a = rng.random((H, W))
    b = rng.random((H, W))
    want = reference(a, b, passes, 1)
    got = simulate(a, b, passes, 1, TW, TH, T, 7, np.random.default_rng(0), exact_margin=1)
    assert not np.array_equal(got, want)
