"""The oracle: CPU restatement of PSkel's iterative stencil path plus a runner
for the reference's own ``runIterativeCPU``.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
package, and only as the checker or the timed CPU baseline. The product
(``pskel_gb300``) never imports it.

* ``pskel_oracle.c`` -> ``_build/libpskel_oracle.so``: the C restatement
  (functions below), pinned bit-for-bit against the reference's outputs in
  ``tests/golden``.
* ``ref_runner.cpp`` -> ``_ref/pskel_ref``: the reference's own
  ``Stencil2D/3D::runIterativeCPU`` built from its headers by ``make_ref.py``.
* ``ref_runner_gpu.cu`` -> ``_ref/pskel_ref_gpu``: the reference's own
  ``Stencil2D::runIterativeGPU`` (one kernel launch per step), the GPU path
  the library is measured beside (``--impl reference`` and a GPU test).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libpskel_oracle.so"
REF_BIN = HERE / "_ref" / "pskel_ref"
REF_GPU_BIN = HERE / "_ref" / "pskel_ref_gpu"

_lib = None


def build() -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "pskel_oracle.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                        "-fvisibility=hidden", str(src), "-o", str(LIB), "-lm"], check=True)
    return LIB


def build_ref() -> Path | None:
    from . import make_ref
    return make_ref.build(require=False)


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _mask2(offsets):
    off = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32).reshape(-1))
    return off, len(offsets)


# ----------------------------------------------------------------- restatement

def lin2d(a_in, a_out, offsets, weights, iters, dtype="f32", rng=0):
    """runIterativeCPU for the weighted linear 2D mask; returns the output array.

    ``a_in``/``a_out`` are copied (the reference clobbers its input). dtype
    "bf16" takes and returns uint16 bit patterns.
    """
    a = np.array(a_in, copy=True, order="C")
    b = np.array(a_out, copy=True, order="C")
    H, W = a.shape
    off, nm = _mask2(offsets)
    L = lib()
    if dtype == "f32":
        wt = np.asarray(weights, dtype=np.float32)
        fn = L.oracle_lin2d_f32
    elif dtype == "f64":
        wt = np.asarray(weights, dtype=np.float64)
        fn = L.oracle_lin2d_f64
    elif dtype == "bf16":
        wt = np.asarray(weights, dtype=np.float32)
        fn = L.oracle_lin2d_bf16
    else:
        raise ValueError(dtype)
    rc = fn(_p(a), _p(b), C.c_long(W), C.c_long(H), C.c_int(nm), _p(off), _p(wt), C.c_long(rng), C.c_long(iters))
    if rc != 0:
        raise ValueError("oracle rejected the grid")
    return b


def life(a_in, a_out, iters, offsets=None, rng=0):
    from pskel_gb300.synth import MOORE8_OFFSETS
    a = np.array(a_in, dtype=np.uint8, copy=True, order="C")
    b = np.array(a_out, dtype=np.uint8, copy=True, order="C")
    H, W = a.shape
    off, nm = _mask2(offsets if offsets is not None else MOORE8_OFFSETS)
    rc = lib().oracle_life(_p(a), _p(b), C.c_long(W), C.c_long(H), C.c_int(nm), _p(off), C.c_long(rng),
                           C.c_long(iters))
    if rc != 0:
        raise ValueError("oracle rejected the grid")
    return b


def advect(a_in, a_out, u, v, iters, K, dt, inv_dx, dtype="f32"):
    npt = {"f32": np.float32, "f64": np.float64, "bf16": np.uint16}[dtype]
    a = np.array(a_in, dtype=npt, copy=True, order="C")
    b = np.array(a_out, dtype=npt, copy=True, order="C")
    uu = np.ascontiguousarray(u, dtype=npt)
    vv = np.ascontiguousarray(v, dtype=npt)
    H, W = a.shape
    fn = {"f32": lib().oracle_advect_f32, "f64": lib().oracle_advect_f64, "bf16": lib().oracle_advect_bf16}[dtype]
    rc = fn(_p(a), _p(b), _p(uu), _p(vv), C.c_long(W), C.c_long(H), C.c_float(K), C.c_float(dt),
            C.c_float(inv_dx), C.c_long(iters))
    if rc != 0:
        raise ValueError("oracle rejected the grid")
    return b


def lin3d(a_in, a_out, offsets, weights, iters, halo=0.0, dtype="f32", every=0):
    """runIterativeCPU for the weighted 3D mask; returns (output, residual norms)."""
    npt = {"f32": np.float32, "f64": np.float64, "bf16": np.uint16}[dtype]
    a = np.array(a_in, dtype=npt, copy=True, order="C")
    b = np.array(a_out, dtype=npt, copy=True, order="C")
    H, W, D = a.shape
    off = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32).reshape(-1))
    nm = len(offsets)
    norms = np.zeros(max(1, iters // every if every else 1), dtype=np.float64)
    if dtype == "f64":
        wt = np.asarray(weights, dtype=np.float64)
        n = lib().oracle_lin3d_f64(_p(a), _p(b), C.c_long(W), C.c_long(H), C.c_long(D), C.c_int(nm), _p(off),
                                   _p(wt), C.c_double(halo), C.c_long(iters), C.c_long(every), _p(norms))
    else:
        wt = np.asarray(weights, dtype=np.float32)
        fn = lib().oracle_lin3d_f32 if dtype == "f32" else lib().oracle_lin3d_bf16
        n = fn(_p(a), _p(b), C.c_long(W), C.c_long(H), C.c_long(D), C.c_int(nm), _p(off), _p(wt),
               C.c_float(halo), C.c_long(iters), C.c_long(every), _p(norms))
    return b, norms[:n]


# ------------------------------------------------------ the reference itself

def have_ref() -> bool:
    return REF_BIN.exists()


def _write_mask(path, offsets, weights):
    with open(path, "w") as f:
        f.write(f"{len(offsets)} {len(offsets[0])}\n")
        for o, w in zip(offsets, weights):
            f.write(" ".join(str(int(x)) for x in o) + " " + float(w).hex() + "\n")


def _run(args, threads):
    env = dict(os.environ)
    env.setdefault("OMP_NUM_THREADS", str(threads))
    out = subprocess.run([str(REF_BIN)] + [str(x) for x in args], check=True, capture_output=True, text=True,
                         env=env)
    return out.stdout


def ref_lin2d(a_in, a_out, offsets, weights, iters, dtype="f32", threads=4):
    npt = {"f32": np.float32, "f64": np.float64, "bf16": np.uint16}[dtype]
    H, W = a_in.shape
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        _write_mask(d / "m.txt", offsets, weights)
        np.ascontiguousarray(a_in, dtype=npt).tofile(d / "in")
        np.ascontiguousarray(a_out, dtype=npt).tofile(d / "out")
        _run(["lin2d", dtype, W, H, iters, threads, d / "m.txt", d / "in", d / "out", d / "res"], threads)
        return np.fromfile(d / "res", dtype=npt).reshape(H, W)


def ref_life(a_in, a_out, iters, threads=4):
    H, W = a_in.shape
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        np.ascontiguousarray(a_in, dtype=np.uint8).tofile(d / "in")
        np.ascontiguousarray(a_out, dtype=np.uint8).tofile(d / "out")
        stdout = _run(["life", W, H, iters, threads, d / "in", d / "out", d / "res"], threads)
        return np.fromfile(d / "res", dtype=np.uint8).reshape(H, W), stdout


def have_ref_gpu() -> bool:
    return REF_GPU_BIN.exists()


def _parse_gpu_run(stdout: str) -> dict:
    """The timed call's lines: the reference's own ``GPU_time <s>`` print
    (copies in and out plus the step loop, PSkelStencil.hpp:1067-1091) and the
    runner's ``{"wall_s", "cell_updates"}`` (the whole call)."""
    import json
    lines = [ln for ln in stdout.splitlines() if ln.strip()]
    info = json.loads(lines[-1])
    gpu_times = [float(ln.split()[1]) for ln in lines if ln.startswith("GPU_time")]
    info["gpu_time_s"] = gpu_times[-1]
    return info


def ref_gpu_life(a_in, a_out, iters, block=(32, 4)):
    """The reference's ``runIterativeGPU`` on the Game of Life: (result, timing).
    The output array is never copied to the device (PSkelStencil.hpp:1071), so
    from the second step on the ring read comes from a fresh device
    allocation: cells within ``iters`` of the edge may differ from the CPU
    path's."""
    H, W = a_in.shape
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        np.ascontiguousarray(a_in, dtype=np.uint8).tofile(d / "in")
        np.ascontiguousarray(a_out, dtype=np.uint8).tofile(d / "out")
        out = subprocess.run([str(REF_GPU_BIN), "life", str(W), str(H), str(iters), str(block[0]), str(block[1]),
                              str(d / "in"), str(d / "out"), str(d / "res")], check=True, capture_output=True,
                             text=True)
        return np.fromfile(d / "res", dtype=np.uint8).reshape(H, W), _parse_gpu_run(out.stdout)


def ref_gpu_lin2d(a_in, a_out, offsets, weights, iters, block=(32, 4)):
    """The reference's ``runIterativeGPU`` on a weighted float32 2D mask:
    (result, timing), with the ring caveat of ``ref_gpu_life``. nvcc contracts
    the weighted sum into FMAs, which round like the separate product and sum
    only when the products are exact (power-of-two weights)."""
    H, W = a_in.shape
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        _write_mask(d / "m.txt", offsets, weights)
        np.ascontiguousarray(a_in, dtype=np.float32).tofile(d / "in")
        np.ascontiguousarray(a_out, dtype=np.float32).tofile(d / "out")
        out = subprocess.run([str(REF_GPU_BIN), "lin2d", str(W), str(H), str(iters), str(block[0]), str(block[1]),
                              str(d / "m.txt"), str(d / "in"), str(d / "out"), str(d / "res")], check=True,
                             capture_output=True, text=True)
        return np.fromfile(d / "res", dtype=np.float32).reshape(H, W), _parse_gpu_run(out.stdout)


def ref_advect(a_in, a_out, u, v, iters, K, dt, inv_dx, dtype="f32", threads=4):
    npt = {"f32": np.float32, "f64": np.float64, "bf16": np.uint16}[dtype]
    H, W = a_in.shape
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        for name, arr in (("in", a_in), ("out", a_out), ("u", u), ("v", v)):
            np.ascontiguousarray(arr, dtype=npt).tofile(d / name)
        _run(["advect", dtype, W, H, iters, threads, repr(float(K)), repr(float(dt)), repr(float(inv_dx)),
              d / "in", d / "out", d / "u", d / "v", d / "res"], threads)
        return np.fromfile(d / "res", dtype=npt).reshape(H, W)


def ref_lin3d(a_in, a_out, offsets, weights, iters, halo=0.0, dtype="f32", every=0, threads=4):
    npt = {"f32": np.float32, "f64": np.float64, "bf16": np.uint16}[dtype]
    H, W, D = a_in.shape
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        _write_mask(d / "m.txt", offsets, weights)
        np.ascontiguousarray(a_in, dtype=npt).tofile(d / "in")
        np.ascontiguousarray(a_out, dtype=npt).tofile(d / "out")
        args = ["lin3d", dtype, W, H, D, iters, threads, d / "m.txt", float(halo).hex(), d / "in", d / "out",
                d / "res"]
        if every:
            args += [every, d / "norms"]
        _run(args, threads)
        res = np.fromfile(d / "res", dtype=npt).reshape(H, W, D)
        norms = np.fromfile(d / "norms", dtype=np.float64) if every else np.zeros(0)
        return res, norms
