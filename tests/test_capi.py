"""C ABI checks that need no GPU: the library loads, exports every symbol
declared in include/*.h, and rejects invalid arguments before touching CUDA."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        for m in re.finditer(r"PSKEL_API\s+[\w\s\*]+?\b(pskel_\w+)\s*\(", h.read_text()):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "pskel_iterate2d" in names and "pskel_run2d_host" in names


def test_library_exports_every_declared_symbol():
    import pskel_gb300 as P
    missing = [n for n in declared_symbols() if not hasattr(P.lib, n)]
    assert not missing, f"not exported: {missing}"


def test_version():
    import pskel_gb300 as P
    assert P.lib.pskel_version() >= 100


def _iterate(st, a, b, W, H, pitch=0, iters=1):
    import pskel_gb300 as P
    return P.lib.pskel_iterate2d(C.byref(st), a, b, W, H, pitch, iters, None, None)


@pytest.mark.parametrize("case", ["null_buf", "same_buf", "empty", "pitch", "neg_iters", "range", "life_mask",
                                  "life_dtype", "lin_u8", "big_mask", "no_weights", "wind", "bad_op", "dim"])
def test_invalid_arguments_rejected_without_gpu(case):
    import pskel_gb300 as P
    from pskel_gb300 import synth as S
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    a, b, W, H, pitch, iters = 0x1000, 0x2000, 64, 64, 0, 3
    expect = P.PSKEL_ERR_INVALID
    if case == "null_buf":
        a = None
    elif case == "same_buf":
        b = a
    elif case == "empty":
        W = 0
    elif case == "pitch":
        pitch = 10
    elif case == "neg_iters":
        iters = -1
    elif case == "range":
        st = P.make_stencil(P.OP_LINEAR, "f32", [(-2, 0), (2, 0)], [0.5, 0.5], rng=1, keep=keep)
    elif case == "life_mask":
        st = P.make_stencil(P.OP_LIFE, "u8", S.JACOBI4_OFFSETS, keep=keep)
        expect = P.PSKEL_ERR_UNSUPPORTED
    elif case == "life_dtype":
        st = P.make_stencil(P.OP_LIFE, "f32", S.MOORE8_OFFSETS, keep=keep)
        expect = P.PSKEL_ERR_UNSUPPORTED
    elif case == "lin_u8":
        st = P.make_stencil(P.OP_LINEAR, "u8", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
        expect = P.PSKEL_ERR_UNSUPPORTED
    elif case == "big_mask":
        off = [(0, i % 5 - 2) for i in range(33)]
        st = P.make_stencil(P.OP_LINEAR, "f32", off, [0.1] * 33, keep=keep)
        expect = P.PSKEL_ERR_UNSUPPORTED
    elif case == "no_weights":
        st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, None, keep=keep)
    elif case == "wind":
        st = P.make_stencil(P.OP_ADVECT, "f32", keep=keep)
    elif case == "bad_op":
        st.op = 7
    elif case == "dim":
        st = P.make_stencil(P.OP_LINEAR, "f32", [(0, 0, 1)], [1.0], keep=keep)
    rc = _iterate(st, a, b, W, H, pitch, iters)
    assert rc == expect, P.lib.pskel_last_error().decode()
    assert P.lib.pskel_last_error().decode() != ""
    assert P.lib.pskel_last_launches2d() == 0  # rejected before any launch


def test_pass_plan_parity():
    # the pass plan must end in the buffer a step-by-step ping-pong ends in
    import pskel_gb300 as P
    buf = (C.c_int32 * 128)()
    for iters in range(0, 70):
        for T in (1, 2, 3, 7, 16):
            n = P.lib.pskel_plan_passes(iters, T, buf, 128)
            p = list(buf[:n])
            assert sum(p) == iters and all(1 <= x <= T for x in p)
            assert all(x % 2 == 1 for x in p)
            assert len(p) % 2 == iters % 2
            if iters >= T:
                assert len(p) <= -(-iters // max(1, T - (T + 1) % 2)) + 1


def test_selftest_rejects_bad_arguments():
    # argument checks come before any device work
    import pskel_gb300 as P
    assert P.lib.pskel_selftest_bounded_wait(4, 10, None) == P.PSKEL_ERR_INVALID
    assert P.lib.pskel_selftest_bounded_wait(-1, 10, None) == P.PSKEL_ERR_INVALID
    assert P.lib.pskel_selftest_bounded_wait(0, 0, None) == P.PSKEL_ERR_INVALID
    assert P.lib.pskel_selftest_bounded_wait(1, (1 << 20) + 1, None) == P.PSKEL_ERR_INVALID


def test_tiled_plan_arithmetic():
    """Slab plan of the out-of-core calls (host only when a slab height or a
    device budget is given): halo = ring + (T-1)*reach rows in 2D, T*reach
    planes in 3D; 2 + ceil(halo/slab) device slots (at least 3) of two
    buffers each, rows 128-byte pitched in 2D, plus both arrays' ring columns
    and ring rows."""
    import pskel_gb300 as P
    from pskel_gb300 import synth as S
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    # 21 steps in passes of at most 7: 7, 7, 7 (20 steps would be 5, 5, 5, 5)
    assert P.tiled_plan(st, (500, 1000), 20, slab_rows=64, inner=7)[1] == 5
    slab, halo, slabs, dev = P.tiled_plan(st, (500, 1000), 21, slab_rows=64, inner=7)
    assert (slab, halo, slabs) == (64, 7, 8)
    sub = 64 + 2 * 7
    up = lambda x: -(-x // 256) * 256  # noqa: E731
    rings = 2 * (up(500 * 2 * 1 * 4) + up(2 * 1 * 4096))
    assert dev == 3 * 2 * up(sub * 4096) + rings
    # slabs thinner than the halo: one more slot per slab the halo spans
    slab, halo, slabs, dev = P.tiled_plan(st, (500, 1000), 21, slab_rows=2, inner=7)
    assert (slab, halo, slabs) == (2, 7, 250)
    assert dev == (2 + 4) * 2 * up((2 + 14) * 4096) + rings
    # budget-sized: rows per slot from the budget, minus the halo on both sides
    slab, halo, slabs, dev = P.tiled_plan(st, (500, 1000), 21, inner=7, device_bytes=4 << 20)
    rows = ((4 << 20) - (rings + (1 << 20))) // (3 * 2 * 4096 + 1000 // 4 + 64)
    assert slab == rows - 2 * 7 and slabs == -(-500 // slab) and dev <= 4 << 20
    # ring wider than the reach: halo = ring + (T-1)*reach
    st3 = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, rng=3, keep=keep)
    assert P.tiled_plan(st3, (500, 1000), 20, slab_rows=10, inner=5)[1] == 3 + 4
    # even inner counts are lowered by one (odd pass lengths keep the ring parity)
    assert P.tiled_plan(st, (500, 1000), 21, slab_rows=10, inner=8)[1] == 7
    # 3D: T * reach planes, no ring columns
    h3 = P.make_stencil(P.OP_LINEAR, "f32", S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, keep=keep)
    slab, halo, slabs, dev = P.tiled_plan(h3, (57, 40, 72), 9, slab_rows=5, inner=3)
    assert (slab, halo, slabs) == (5, 3, 12)
    assert dev == 3 * 2 * (-(-(5 + 6) * 40 * 72 * 4 // 256) * 256)


def test_tiled_rejects_bad_arguments():
    import ctypes as C

    import numpy as np

    import pskel_gb300 as P
    from pskel_gb300 import synth as S
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    a = np.zeros((40, 50), np.float32)
    b = np.zeros((40, 50), np.float32)
    f = P.lib.pskel_run2d_host_tiled
    assert f(C.byref(st), None, b.ctypes.data, 50, 40, 3, 8, 3, 0, None) == P.PSKEL_ERR_INVALID
    assert f(C.byref(st), a.ctypes.data, a.ctypes.data, 50, 40, 3, 8, 3, 0, None) == P.PSKEL_ERR_INVALID
    assert f(C.byref(st), a.ctypes.data, b.ctypes.data, 50, 40, -1, 8, 3, 0, None) == P.PSKEL_ERR_INVALID
    out = (C.c_int64 * 4)()
    assert P.lib.pskel_tiled_plan(C.byref(st), 50, 40, 1, 3, -2, 3, 0, out) == P.PSKEL_ERR_INVALID
    assert P.lib.pskel_tiled_plan(C.byref(st), 50, 40, 1, 3, 0, -1, 1 << 20, out) == P.PSKEL_ERR_INVALID
    # a budget too small for one row plus its halo
    assert P.lib.pskel_tiled_plan(C.byref(st), 50000, 40, 1, 30, 0, 15, 2 << 20, out) == P.PSKEL_ERR_NOMEM
    life = P.make_stencil(P.OP_LIFE, "f32", S.MOORE8_OFFSETS, keep=keep)
    assert P.lib.pskel_tiled_plan(C.byref(life), 50, 40, 1, 3, 8, 3, 0, out) == P.PSKEL_ERR_UNSUPPORTED
