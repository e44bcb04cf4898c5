"""pskel_gb300: GB300-native iterative stencils behind PSkel's API.

This Python module is a thin ctypes binding of the C ABI in
``include/pskel_gb300.h`` (the library ``pskel_gb300/libpskel_gb300.so``),
used by the tests and the benchmark. C++ applications use the drop-in headers
``include/PSkel*.h`` instead. There is no CPU fallback: every call runs the
CUDA kernels of the library. The library is opened on first use (so that
the seeded input generators in ``pskel_gb300.synth`` import without it), and
that first use raises if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libpskel_gb300.so"

PSKEL_OK, PSKEL_ERR_INVALID, PSKEL_ERR_UNSUPPORTED, PSKEL_ERR_CUDA, PSKEL_ERR_DEVICE, PSKEL_ERR_NOMEM = range(6)
U8, F32, BF16 = 0, 1, 2
OP_LINEAR, OP_LIFE, OP_ADVECT = 0, 1, 2
_DTYPES = {"u8": U8, "f32": F32, "bf16": BF16}
_ESIZE = {U8: 1, F32: 4, BF16: 2}


class PskelError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"pskel status {status}: {msg}")
        self.status = status


class Mask(C.Structure):
    _fields_ = [("size", C.c_int32), ("dimension", C.c_int32), ("offsets", C.POINTER(C.c_int32)),
                ("weights", C.POINTER(C.c_float)), ("halo_value", C.c_float), ("range", C.c_int32)]


class Stencil(C.Structure):
    _fields_ = [("op", C.c_int), ("dtype", C.c_int), ("mask", Mask), ("wind_u", C.c_void_p),
                ("wind_v", C.c_void_p), ("diffusivity", C.c_float), ("dt", C.c_float), ("inv_dx", C.c_float)]


class Schedule(C.Structure):
    _fields_ = [("tile_w", C.c_int32), ("tile_h", C.c_int32), ("tile_d", C.c_int32), ("time_steps", C.c_int32),
                ("ctas", C.c_int32)]


class BatchGrid(C.Structure):
    _fields_ = [("in_", C.c_void_p), ("out", C.c_void_p), ("width", C.c_int64), ("height", C.c_int64),
                ("pitch", C.c_int64), ("iterations", C.c_int64), ("schedule", Schedule)]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    lib.pskel_version.restype = C.c_int32
    lib.pskel_last_error.restype = C.c_char_p
    lib.pskel_last_launches2d.restype = C.c_int64
    lib.pskel_last_launches2d.argtypes = []
    lib.pskel_sync.argtypes = [C.c_void_p]
    lib.pskel_iterate2d.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                    C.c_int64, C.POINTER(Schedule), C.c_void_p]
    lib.pskel_plan_passes.argtypes = [C.c_int64, C.c_int32, C.POINTER(C.c_int32), C.c_int32]
    lib.pskel_plan_passes.restype = C.c_int32
    lib.pskel_run2d_host.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                     C.POINTER(Schedule)]
    lib.pskel_iterate3d.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                    C.c_int64, C.POINTER(Schedule), C.c_int64, C.c_void_p, C.c_void_p]
    lib.pskel_batch_create.argtypes = [C.POINTER(Stencil), C.POINTER(BatchGrid), C.c_int32, C.POINTER(C.c_void_p)]
    lib.pskel_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    lib.pskel_batch_cell_updates.argtypes = [C.c_void_p]
    lib.pskel_batch_cell_updates.restype = C.c_int64
    lib.pskel_batch_destroy.argtypes = [C.c_void_p]
    lib.pskel_iterate3d_noalloc.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                            C.c_int64, C.c_int64, C.POINTER(Schedule), C.c_int64, C.c_void_p,
                                            C.c_void_p]
    lib.pskel_selftest_bounded_wait.argtypes = [C.c_int32, C.c_uint32, C.c_void_p]
    lib.pskel_run3d_host.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                     C.c_int64, C.POINTER(Schedule), C.c_int64, C.c_void_p]
    lib.pskel_run2d_host_tiled.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                           C.c_int64, C.c_int64, C.c_int32, C.c_int64, C.POINTER(Schedule)]
    lib.pskel_run3d_host_tiled.argtypes = [C.POINTER(Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                           C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int64, C.POINTER(Schedule)]
    lib.pskel_tiled_plan.argtypes = [C.POINTER(Stencil), C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                     C.c_int32, C.c_int64, C.POINTER(C.c_int64)]
    return lib


class _Lib:
    """The library, opened on first use: importing the package (for example
    only for ``pskel_gb300.synth``, the seeded input generators) maps no
    native code, and the first call raises ImportError if the library has not
    been built -- there is no other path to fall back to."""

    _cdll = None

    def __getattr__(self, name):
        if _Lib._cdll is None:
            _Lib._cdll = _load()
        return getattr(_Lib._cdll, name)


lib = _Lib()


def load():
    """Opens the library now (raises ImportError if it is missing)."""
    lib.pskel_version()
    return _Lib._cdll


def _check(status: int):
    if status != PSKEL_OK:
        raise PskelError(status, lib.pskel_last_error().decode())


class _Keep:
    """Holds the ctypes arrays a descriptor points to for the call's duration."""

    def __init__(self):
        self.refs = []


def make_mask(offsets, weights=None, halo=0.0, rng=0, keep: _Keep | None = None) -> Mask:
    offsets = [tuple(o) for o in offsets]
    dim = len(offsets[0]) if offsets else 2
    off = (C.c_int32 * (len(offsets) * dim))(*[int(x) for o in offsets for x in o])
    m = Mask(size=len(offsets), dimension=dim, offsets=C.cast(off, C.POINTER(C.c_int32)), halo_value=float(halo),
             range=int(rng))
    if keep is not None:
        keep.refs.append(off)
    if weights is not None:
        wt = (C.c_float * len(weights))(*[float(w) for w in weights])
        m.weights = C.cast(wt, C.POINTER(C.c_float))
        if keep is not None:
            keep.refs.append(wt)
    return m


def make_stencil(op: int, dtype: str, offsets=(), weights=None, halo=0.0, rng=0, wind=(None, None), K=0.0, dt=0.0,
                 inv_dx=0.0, keep: _Keep | None = None) -> Stencil:
    st = Stencil(op=op, dtype=_DTYPES[dtype])
    if offsets:
        st.mask = make_mask(offsets, weights, halo, rng, keep)
    else:
        st.mask = Mask(size=0, dimension=2)
    st.wind_u, st.wind_v = wind
    st.diffusivity, st.dt, st.inv_dx = K, dt, inv_dx
    return st


def make_schedule(sched) -> Schedule | None:
    if sched is None:
        return None
    if isinstance(sched, Schedule):
        return sched
    return Schedule(**sched)


def _ptr(t):
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def iterate2d(st: Stencil, a_in, a_out, iterations: int, sched=None, pitch: int = 0, stream=None, width=None,
              height=None):
    """Device-buffer run (torch CUDA tensors or raw pointers). Asynchronous."""
    H = height if height is not None else a_in.shape[0]
    W = width if width is not None else a_in.shape[1]
    sc = make_schedule(sched)
    _check(lib.pskel_iterate2d(C.byref(st), _ptr(a_in), _ptr(a_out), W, H, pitch, iterations,
                               C.byref(sc) if sc is not None else None, stream))


def sync(stream=None):
    _check(lib.pskel_sync(stream))


def run2d_host(st: Stencil, a_in: np.ndarray, a_out: np.ndarray, iterations: int, sched=None):
    """runIterativeGPU on host arrays: returns the output array (a_out is updated in place)."""
    assert a_in.flags.c_contiguous and a_out.flags.c_contiguous
    H, W = a_in.shape
    sc = make_schedule(sched)
    _check(lib.pskel_run2d_host(C.byref(st), a_in.ctypes.data, a_out.ctypes.data, W, H, iterations,
                                C.byref(sc) if sc is not None else None))
    return a_out


def iterate3d(st: Stencil, a_in, a_out, iterations: int, sched=None, residual_every: int = 0, residuals=None,
              stream=None):
    """Device-buffer 3D run; arrays are [H][W][D] (d fastest). Asynchronous."""
    H, W, D = a_in.shape
    sc = make_schedule(sched)
    _check(lib.pskel_iterate3d(C.byref(st), _ptr(a_in), _ptr(a_out), W, H, D, iterations,
                               C.byref(sc) if sc is not None else None, residual_every, _ptr(residuals), stream))


def run3d_host(st: Stencil, a_in: np.ndarray, a_out: np.ndarray, iterations: int, sched=None, residual_every=0):
    """Stencil3D::runIterativeGPU on host arrays; returns (output, residual norms)."""
    assert a_in.flags.c_contiguous and a_out.flags.c_contiguous
    H, W, D = a_in.shape
    n = iterations // residual_every if residual_every > 0 else 0
    res = np.zeros(max(n, 1), dtype=np.float64)
    sc = make_schedule(sched)
    _check(lib.pskel_run3d_host(C.byref(st), a_in.ctypes.data, a_out.ctypes.data, W, H, D, iterations,
                                C.byref(sc) if sc is not None else None, residual_every, res.ctypes.data))
    return a_out, res[:n]


def run2d_host_tiled(st: Stencil, a_in: np.ndarray, a_out: np.ndarray, iterations: int, slab_rows: int = 0,
                     inner: int = 0, device_bytes: int = 0, sched=None):
    """Out-of-core 2D run: slabs of rows streamed host -> device -> host; a_out is updated in place."""
    assert a_in.flags.c_contiguous and a_out.flags.c_contiguous
    H, W = a_in.shape
    sc = make_schedule(sched)
    _check(lib.pskel_run2d_host_tiled(C.byref(st), a_in.ctypes.data, a_out.ctypes.data, W, H, iterations, slab_rows,
                                      inner, device_bytes, C.byref(sc) if sc is not None else None))
    return a_out


def run3d_host_tiled(st: Stencil, a_in: np.ndarray, a_out: np.ndarray, iterations: int, slab_planes: int = 0,
                     inner: int = 0, device_bytes: int = 0, sched=None):
    """Out-of-core 3D run over h-plane slabs; arrays are [H][W][D]; a_out is updated in place."""
    assert a_in.flags.c_contiguous and a_out.flags.c_contiguous
    H, W, D = a_in.shape
    sc = make_schedule(sched)
    _check(lib.pskel_run3d_host_tiled(C.byref(st), a_in.ctypes.data, a_out.ctypes.data, W, H, D, iterations,
                                      slab_planes, inner, device_bytes, C.byref(sc) if sc is not None else None))
    return a_out


def tiled_plan(st: Stencil, shape, iterations: int, slab_rows: int = 0, inner: int = 0, device_bytes: int = 0):
    """(core rows per slab, halo rows, slabs per pass, device bytes) of an out-of-core run."""
    H, W = shape[0], shape[1]
    D = shape[2] if len(shape) == 3 else 1
    out = (C.c_int64 * 4)()
    _check(lib.pskel_tiled_plan(C.byref(st), W, H, D, iterations, slab_rows, inner, device_bytes, out))
    return tuple(out)


class Batch:
    """Many 2D grids in one persistent launch (a CUDA graph). `grids` is a list
    of (in, out, iterations, time_steps) with torch CUDA tensors [H][W] or
    (in, out, iterations, time_steps, pitch)."""

    def __init__(self, st: Stencil, grids):
        arr = (BatchGrid * len(grids))()
        for i, g in enumerate(grids):
            a, b, iters, T = g[:4]
            pitch = g[4] if len(g) > 4 else 0
            arr[i].in_ = _ptr(a)
            arr[i].out = _ptr(b)
            arr[i].height, arr[i].width = a.shape[0], (g[5] if len(g) > 5 else a.shape[1])
            arr[i].pitch = pitch
            arr[i].iterations = iters
            arr[i].schedule = Schedule(time_steps=T)
        self._st = st
        self.handle = C.c_void_p()
        _check(lib.pskel_batch_create(C.byref(st), arr, len(grids), C.byref(self.handle)))

    def run(self, stream=None):
        _check(lib.pskel_batch_run(self.handle, stream))

    @property
    def cell_updates(self) -> int:
        return lib.pskel_batch_cell_updates(self.handle)

    def close(self):
        if self.handle:
            lib.pskel_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
