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
    assert P.lib.pskel_selftest_bounded_wait(2, 10, None) == P.PSKEL_ERR_INVALID
    assert P.lib.pskel_selftest_bounded_wait(0, 0, None) == P.PSKEL_ERR_INVALID
    assert P.lib.pskel_selftest_bounded_wait(1, (1 << 20) + 1, None) == P.PSKEL_ERR_INVALID
