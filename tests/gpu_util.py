"""Helpers for the GPU parity tests: run the library on torch CUDA buffers."""
from __future__ import annotations

import numpy as np

import pskel_gb300 as P


def to_dev(torch, a: np.ndarray, pitch: int | None = None):
    """Copy a 2D host array to a CUDA tensor, optionally with a wider row pitch."""
    if pitch is None or pitch == a.shape[1]:
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()
    buf = np.zeros((a.shape[0], pitch), dtype=a.dtype)
    buf[:, : a.shape[1]] = a
    return torch.from_numpy(buf).cuda()


def from_dev(t, width: int) -> np.ndarray:
    return t.cpu().numpy()[:, :width].copy()


def np_view(a: np.ndarray, dtype: str) -> np.ndarray:
    """bf16 grids travel as uint16 bit patterns; torch holds them as int16."""
    return a.view(np.int16) if dtype == "bf16" else a


def aligned_pitch(W: int, esize: int) -> int:
    """Row pitch (elements) rounded up to 16 bytes, as the TMA path needs."""
    return -(-W * esize // 16) * 16 // esize


def run2d(torch, st, a_in, a_out, iters, sched=None, pitch="aligned", dtype="f32"):
    """Run iterate2d on device copies; return the result array (host).

    The default row pitch is 16-byte aligned (tiles staged by TMA); an explicit
    pitch may be unaligned (tiles staged by plain loads)."""
    H, W = a_in.shape
    if pitch == "aligned":
        pitch = aligned_pitch(W, a_in.dtype.itemsize)
    x = to_dev(torch, np_view(a_in, dtype), pitch)
    y = to_dev(torch, np_view(a_out, dtype), pitch)
    P.iterate2d(st, x, y, iters, sched=sched, pitch=pitch or 0, width=W, height=H)
    P.sync()
    res = from_dev(y if iters % 2 == 1 else x, W)
    return res.view(np.uint16) if dtype == "bf16" else res


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)
