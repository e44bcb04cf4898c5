"""The no-allocation 3D entry point (pskel_iterate3d_noalloc) against the
regular one (pskel_iterate3d).

It exists for callers that cannot let the library call cudaMalloc: a host
application that owns all device memory through its own pool, or a
latency-critical loop that cannot absorb cudaMalloc's implicit
synchronisation. Its scratch lives in a fixed-size file-scope device array.
This file is collected last so that a failure here comes after every other
test has run; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import pskel_gb300 as P
from pskel_gb300 import synth as S

pytestmark = pytest.mark.gpu


def _case(torch, seed, shape=(48, 37, 64)):
    H, W, D = shape
    a = S.uniform_f32(seed, 1, (H, W, D))
    x = torch.from_numpy(a).cuda()
    y = torch.zeros_like(x)
    return x, y


def _call(fn, torch, st, x, y, iters, every, sched):
    n = iters // every
    res = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
    H, W, D = x.shape
    rc = fn(C.byref(st), x.data_ptr(), y.data_ptr(), W, H, D, iters, C.byref(sched), every, res.data_ptr(), None)
    assert rc == P.PSKEL_OK, P.lib.pskel_last_error().decode()
    torch.cuda.synchronize()
    out = (y if iters % 2 == 1 else x).clone()
    return out, res[:n].clone()


def test_noalloc_matches_regular_entry_point_twice(cuda):
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, halo=0.25, keep=keep)
    sched = P.Schedule(time_steps=2, tile_w=16, tile_h=0, tile_d=32, ctas=0)
    for call, seed in enumerate((3, 4)):  # two calls in a row: no state may leak between them
        iters, every = 9, 3
        x0, y0 = _case(torch, seed)
        want, want_res = _call(P.lib.pskel_iterate3d, torch, st, x0.clone(), y0.clone(), iters, every, sched)
        got, got_res = _call(P.lib.pskel_iterate3d_noalloc, torch, st, x0.clone(), y0.clone(), iters, every, sched)
        assert torch.equal(got, want), f"call {call}: grids differ"
        # same kernels, same schedule, same reduction order: the norms agree to
        # the residual tolerance of the 3D tests (they are in fact identical)
        np.testing.assert_allclose(got_res.cpu().numpy(), want_res.cpu().numpy(), rtol=1e-12, atol=0)
        assert got_res.shape[0] == iters // every


def test_noalloc_default_streaming_path_allocates_nothing(cuda):
    """The schedule callers get by default: the one-step TMA streaming kernel
    (7-point cross) with a residual every 10 steps, 50 steps on 64^3. Two
    calls in a row match the regular entry point; once both entry points have
    run (the first no-allocation call on a device looks up its arrays'
    addresses, and the kernels load on first use), further calls leave the
    device's free memory unchanged."""
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, keep=keep)
    default = P.Schedule(time_steps=0, tile_w=0, tile_h=0, tile_d=0, ctas=0)
    iters, every = 50, 10
    shape = (64, 64, 64)
    H, W, D = shape
    res = torch.zeros(iters // every, dtype=torch.float64, device="cuda")

    def noalloc(x, y):
        rc = P.lib.pskel_iterate3d_noalloc(C.byref(st), x.data_ptr(), y.data_ptr(), W, H, D, iters, None, every,
                                           res.data_ptr(), None)
        assert rc == P.PSKEL_OK, P.lib.pskel_last_error().decode()

    for call, seed in enumerate((11, 12)):
        x0, y0 = _case(torch, seed, shape)
        x, y = x0.clone(), y0.clone()
        noalloc(x, y)
        got, got_res = (y if iters % 2 else x).clone(), res.clone()
        want, want_res = _call(P.lib.pskel_iterate3d, torch, st, x0.clone(), y0.clone(), iters, every, default)
        assert torch.equal(got, want), f"call {call}: grids differ"
        np.testing.assert_allclose(got_res.cpu().numpy(), want_res.cpu().numpy(), rtol=1e-12, atol=0)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        noalloc(x, y)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, f"free device memory changed across calls: {free_before} -> {free_after}"


def test_noalloc_rejects_scratch_beyond_its_capacity(cuda):
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, keep=keep)
    # 8 fused steps on 4096 CTAs need 32768 partial sums, above the 16384 cap
    sched = P.Schedule(time_steps=8, tile_w=1, tile_h=0, tile_d=8, ctas=4096)
    x = torch.zeros((16, 512, 512), dtype=torch.float32, device="cuda")
    y = torch.zeros_like(x)
    res = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = P.lib.pskel_iterate3d_noalloc(C.byref(st), x.data_ptr(), y.data_ptr(), 512, 16, 512, 8, C.byref(sched), 2,
                                       res.data_ptr(), None)
    assert rc == P.PSKEL_ERR_UNSUPPORTED
    assert "capacity" in P.lib.pskel_last_error().decode()
