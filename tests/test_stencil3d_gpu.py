"""3D stencils on the GPU against the oracle.

fp32 and bf16-storage grids are compared bit for bit (same operation order,
no contraction, bf16 rounding every step). The fp64 residual norms are
compared with a relative tolerance of 1e-12 plus the worst-case error of the
oracle's own serial fp64 sum over n cells (n * 2^-53): the kernel adds per-CTA
partials in a fixed tree, which is more accurate than the serial loop.
"""
from __future__ import annotations

import numpy as np
import pytest

import pskel_gb300 as P
from pskel_gb300 import synth as S
from tests.gpu_util import bits

pytestmark = pytest.mark.gpu

RES_RTOL = 1e-12


def res_rtol(shape) -> float:
    return RES_RTOL + float(np.prod(shape)) * 2.0**-53


def grids(W, H, D, seed, dtype):
    a, _ = S.heat3d(W, H, D, seed=seed)
    b = S.uniform_f32(seed + 50, S.S_GRID, a.shape)  # the output's initial contents are never read
    if dtype == "bf16":
        return S.f32_to_bf16(a), S.f32_to_bf16(b)
    return a, b


def run3d(torch, st, a, b, iters, sched=None, every=0, dtype="f32"):
    view = (lambda x: x.view(np.int16)) if dtype == "bf16" else (lambda x: x)
    x = torch.from_numpy(view(np.ascontiguousarray(a))).cuda()
    y = torch.from_numpy(view(np.ascontiguousarray(b))).cuda()
    n = iters // every if every else 0
    res = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
    P.iterate3d(st, x, y, iters, sched=sched, residual_every=every, residuals=res if every else None)
    P.sync()
    out = (y if iters % 2 == 1 else x).cpu().numpy()
    if dtype == "bf16":
        out = out.view(np.uint16)
    return out, res.cpu().numpy()[:n]


def heat(keep, dtype="f32", halo=0.0):
    return P.make_stencil(P.OP_LINEAR, dtype, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, halo=halo, keep=keep)


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("W,H,D", [(11, 9, 13), (32, 17, 64), (40, 33, 72), (1, 1, 1), (70, 5, 8)])
@pytest.mark.parametrize("iters", [1, 2, 5])
def test_heat3d_matches_oracle(cuda, oracle_mod, dtype, W, H, D, iters):
    keep = P._Keep()
    a, b = grids(W, H, D, W + H + D, dtype)
    got, res = run3d(cuda, heat(keep, dtype, halo=0.5), a, b, iters, every=2, dtype=dtype)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=0.5, dtype=dtype, every=2)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=RES_RTOL, atol=0)


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("W,H,D", [(40, 33, 72), (17, 50, 264), (300, 7, 8)])
@pytest.mark.parametrize("th,ctas", [(0, 0), (3, 1), (64, 5), (1, 0)])
@pytest.mark.parametrize("halo", [0.0, -0.0, 0.1])
def test_heat3d_streaming_items(cuda, oracle_mod, dtype, W, H, D, th, ctas, halo):
    # one step per launch (planes staged by TMA): ragged blocks in w and d,
    # work items of th planes, few persistent blocks (every block runs many
    # items through its plane ring); +0.0 is the zero-filled halo, -0.0 the
    # substituted one, 0.1 (not a bf16 value) takes the generic kernel for bf16
    keep = P._Keep()
    a, b = grids(W, H, D, W * H + D, dtype)
    sch = dict(time_steps=1, tile_w=0, tile_h=th, tile_d=0, ctas=ctas)
    got, res = run3d(cuda, heat(keep, dtype, halo=halo), a, b, 6, sched=sch, every=3, dtype=dtype)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 6, halo=halo, dtype=dtype, every=3)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=RES_RTOL, atol=0)


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("W,H,D", [(40, 33, 72), (17, 50, 264), (300, 7, 8), (16, 3, 256)])
@pytest.mark.parametrize("th,ctas", [(0, 0), (3, 1), (64, 5), (1, 0)])
@pytest.mark.parametrize("halo", [0.0, -0.0, 0.5])
@pytest.mark.parametrize("iters,every", [(6, 3), (7, 1), (9, 0)])
def test_heat3d_two_step_streaming(cuda, oracle_mod, dtype, W, H, D, th, ctas, halo, iters, every):
    # two steps per launch (stream3d_tb.cu): the second step fused behind the
    # first in shared memory; ragged w and d blocks, work items of th planes,
    # few persistent blocks; residuals reported by either step of a pass (and
    # by both, every=1); even and odd iteration counts (an even number of
    # two-step passes, the rest one-step passes)
    keep = P._Keep()
    a, b = grids(W, H, D, W * H + D + iters, dtype)
    sch = dict(time_steps=2, tile_w=0, tile_h=th, tile_d=0, ctas=ctas)
    got, res = run3d(cuda, heat(keep, dtype, halo=halo), a, b, iters, sched=sch, every=every, dtype=dtype)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=halo, dtype=dtype, every=every)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=res_rtol(a.shape), atol=0)


# weights whose products round: a product fused with the following sum into
# one multiply-add would change the last bit (the heat weights 1/4, 1/8 are
# exact, so a fused and an unfused product agree there)
INEXACT7 = [0.31, 0.07, 0.11, 0.13, 0.17, 0.09, 0.12]


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("T", [1, 2])
@pytest.mark.parametrize("halo", [0.0, 0.5])
@pytest.mark.parametrize("W,H,D", [(70, 37, 264), (17, 50, 40)])
def test_cross7_inexact_weights(cuda, oracle_mod, dtype, T, halo, W, H, D):
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.HEAT7_OFFSETS, INEXACT7, halo=halo, keep=keep)
    a, b = grids(W, H, D, W + T, dtype)
    sch = dict(time_steps=T, tile_w=0, tile_h=0, tile_d=0, ctas=0)
    got, res = run3d(cuda, st, a, b, 9, sched=sch, every=3, dtype=dtype)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, INEXACT7, 9, halo=halo, dtype=dtype, every=3)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=res_rtol(a.shape), atol=0)


@pytest.mark.parametrize("T,tw,td,th", [(1, 0, 0, 0), (2, 16, 32, 0), (3, 8, 16, 5), (4, 32, 64, 7), (8, 8, 8, 0),
                                        (2, 0, 0, 1), (3, 16, 16, 13)])
def test_heat3d_schedules(cuda, oracle_mod, T, tw, td, th):
    # th: output planes per work item along h (chunks with warm-up planes)
    keep = P._Keep()
    a, b = grids(48, 31, 40, T, "f32")
    sch = dict(time_steps=T, tile_w=tw, tile_h=th, tile_d=td, ctas=0)
    got, res = run3d(cuda, heat(keep), a, b, 13, sched=sch, every=3)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 13, dtype="f32", every=3)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=RES_RTOL, atol=0)


def test_general_3d_mask_radius2(cuda, oracle_mod):
    keep = P._Keep()
    off = [(0, 0, 0), (-2, 0, 0), (1, 1, 0), (0, -1, 2), (0, 0, -2), (2, -2, 1), (-1, 0, 1), (1, 0, -1), (0, 2, 0)]
    wt = [0.3, 0.1, 0.05, 0.1, 0.15, 0.05, 0.1, 0.07, 0.08]
    st = P.make_stencil(P.OP_LINEAR, "f32", off, wt, halo=-0.25, keep=keep)
    a, b = grids(37, 23, 48, 3, "f32")
    for iters in (1, 4, 7):
        got, _ = run3d(cuda, st, a, b, iters)
        want, _ = oracle_mod.lin3d(a, b, off, wt, iters, halo=-0.25)
        assert np.array_equal(bits(got), bits(want))


def test_heat3d_host_entry_point(cuda, oracle_mod):
    keep = P._Keep()
    for dtype in ("f32", "bf16"):
        a, b = grids(64, 40, 64, 9, dtype)
        a0 = a.copy()
        out, res = P.run3d_host(heat(keep, dtype), a, b.copy(), 10, residual_every=5)
        want, wres = oracle_mod.lin3d(a0, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 10, dtype=dtype, every=5)
        assert np.array_equal(bits(out), bits(want))
        np.testing.assert_allclose(res, wres, rtol=RES_RTOL, atol=0)
        assert np.array_equal(a, a0)


def test_heat3d_c4_size_vs_oracle_and_fp64_error(cuda, oracle_mod):
    # 512^3: 10 steps against the fp32 oracle (and its residual), then the
    # full 50 steps checked for schedule invariance, with the fp32 and bf16
    # errors against the fp64 oracle on a 128^3 cut reported.
    keep = P._Keep()
    a, b = grids(512, 512, 512, 1, "f32")
    got, res = run3d(cuda, heat(keep), a, b, 10, every=10)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 10, every=10)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=res_rtol(a.shape), atol=0)
    r2, n2 = run3d(cuda, heat(keep), a, b, 50, every=10, sched=dict(time_steps=2, tile_w=0, tile_h=0, tile_d=0, ctas=0))
    r3, n3 = run3d(cuda, heat(keep), a, b, 50, every=10, sched=dict(time_steps=3, tile_w=16, tile_h=0, tile_d=32,
                                                                     ctas=0))
    r1, n1 = run3d(cuda, heat(keep), a, b, 50, every=10)  # default: one step per launch, streaming kernel
    assert np.array_equal(bits(r2), bits(r3))
    assert np.array_equal(bits(r1), bits(r2))
    np.testing.assert_allclose(n2, n3, rtol=RES_RTOL, atol=0)
    np.testing.assert_allclose(n1, n2, rtol=RES_RTOL, atol=0)
    assert np.all(np.diff(n2) < 0), "the heat equation's residual must decay"
    c, d = grids(128, 128, 128, 2, "f32")
    g32, _ = run3d(cuda, heat(keep), c, d, 50)
    gb, _ = run3d(cuda, heat(keep, "bf16"), S.f32_to_bf16(c), S.f32_to_bf16(d), 50, dtype="bf16")
    ref64, _ = oracle_mod.lin3d(c.astype(np.float64), d.astype(np.float64), S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 50,
                                dtype="f64")
    e32 = float(np.max(np.abs(g32 - ref64)))
    eb = float(np.max(np.abs(S.bf16_to_f32(gb) - ref64)))
    print(f"\nFP64-ERROR heat3d 128^3 x50: max abs fp32 {e32:.3e}, bf16 storage {eb:.3e}")
    assert e32 < 1e-5 and eb < 0.05


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("W,H,D", [(40, 200, 64), (24, 128, 32), (17, 300, 16)])
@pytest.mark.parametrize("iters,every", [(2, 0), (7, 3), (16, 4), (65, 13)])
@pytest.mark.parametrize("halo", [0.0, 0.5])
def test_host_run_wavefront(cuda, oracle_mod, dtype, W, H, D, iters, every, halo):
    """pskel_run3d_host on grids of 128+ planes: chunks of planes are copied in
    while earlier planes compute, and final planes go back while later ones
    compute (a wavefront over the chunks). Same bits as the oracle; the fp64
    residual norms within the stated tolerance."""
    keep = P._Keep()
    a, b = grids(W, H, D, W + H + D + iters, dtype)
    st = heat(keep, dtype, halo=halo)
    got, res = P.run3d_host(st, np.ascontiguousarray(a), np.ascontiguousarray(b).copy(), iters, residual_every=every)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=halo, dtype=dtype, every=every)
    assert np.array_equal(bits(got), bits(want))
    if every:
        np.testing.assert_allclose(res, wres, rtol=res_rtol(a.shape), atol=0)


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
@pytest.mark.parametrize("iters,every", [(41, 5), (38, 0), (33, 1)])
@pytest.mark.parametrize("halo", [0.0, 0.5])
def test_host_run_wavefront_two_step_middle(cuda, oracle_mod, dtype, iters, every, halo):
    """Two steps per pass (fp32's default, or asked for): the host call's
    middle steps run as pairs of two-step passes between the band wavefronts,
    with residual steps inside the pairs; weights whose products round."""
    keep = P._Keep()
    a, b = grids(40, 150, 64, iters + 7, dtype)
    st = P.make_stencil(P.OP_LINEAR, dtype, S.HEAT7_OFFSETS, INEXACT7, halo=halo, keep=keep)
    got, res = P.run3d_host(st, np.ascontiguousarray(a), np.ascontiguousarray(b).copy(), iters,
                            sched=dict(time_steps=2, tile_w=0, tile_h=0, tile_d=0, ctas=0), residual_every=every)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, INEXACT7, iters, halo=halo, dtype=dtype, every=every)
    assert np.array_equal(bits(got), bits(want))
    if every:
        np.testing.assert_allclose(res, wres, rtol=res_rtol(a.shape), atol=0)


def test_host_run_wavefront_max_iterations(cuda, oracle_mod):
    keep = P._Keep()
    a, b = grids(32, 160, 32, 5, "f32")
    got, res = P.run3d_host(heat(keep), a, b.copy(), 256, residual_every=64)
    want, wres = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, 256, dtype="f32", every=64)
    assert np.array_equal(bits(got), bits(want))
    np.testing.assert_allclose(res, wres, rtol=res_rtol(a.shape), atol=0)
