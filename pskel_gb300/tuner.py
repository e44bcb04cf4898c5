"""Schedule search for the 2D stencils (bindings of the C ABI's tuner and
cost-model entry points).

* ``exhaustive``     -- time every candidate schedule on the GPU, keep the
                        fastest (the measured replacement of the reference's
                        runIterativeAutoGPU search, PSkelStencil.hpp:2007-2076);
* ``ga_schedule``    -- the reference's GA with its analytic objective
                        (PSkelStencil.hpp:1883-1941), no timing;
* ``CostModel``      -- the MLP (library CUDA kernels for forward, backward and
                        Adam) trained on the exhaustive tuner's timings; it
                        ranks candidates by predicted log time.

A schedule only changes speed: every candidate gives bit-identical results.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

import pskel_gb300 as P

NFEAT = 11


def _setup():
    L = P.lib
    L.pskel_candidates2d.argtypes = [C.POINTER(P.Stencil), C.c_int64, C.c_int64, C.c_int64, C.POINTER(P.Schedule),
                                     C.c_int32]
    L.pskel_candidates2d.restype = C.c_int32
    L.pskel_time2d.argtypes = [C.POINTER(P.Stencil), C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                               C.c_int64, C.POINTER(P.Schedule), C.c_int32, C.c_int32, C.POINTER(C.c_double),
                               C.c_void_p]
    L.pskel_time_batch2d.argtypes = [C.POINTER(P.Stencil), C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                     C.POINTER(P.Schedule), C.c_int32, C.c_int32, C.POINTER(C.c_double),
                                     C.POINTER(C.c_int32), C.c_void_p]
    L.pskel_ga_schedule2d.argtypes = [C.POINTER(P.Stencil), C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_int32,
                                      C.c_int32, C.POINTER(P.Schedule), C.POINTER(C.c_double)]
    L.pskel_schedule_features2d.argtypes = [C.POINTER(P.Stencil), C.c_int64, C.c_int64, C.c_int64,
                                            C.POINTER(P.Schedule), C.POINTER(C.c_float)]
    L.pskel_schedule_features2d.restype = C.c_int32
    L.pskel_auto_schedule2d.argtypes = [C.POINTER(P.Stencil), C.c_int64, C.c_int64, C.c_int64, C.POINTER(P.Schedule)]
    L.pskel_mlp_create.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]
    L.pskel_mlp_num_params.argtypes = [C.c_void_p]
    L.pskel_mlp_num_params.restype = C.c_int64
    L.pskel_mlp_get_params.argtypes = [C.c_void_p, C.c_void_p]
    L.pskel_mlp_set_params.argtypes = [C.c_void_p, C.c_void_p]
    L.pskel_mlp_predict.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
    L.pskel_mlp_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_float)]
    L.pskel_mlp_train.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_float,
                                  C.POINTER(C.c_float)]
    L.pskel_mlp_save.argtypes = [C.c_void_p, C.c_char_p]
    L.pskel_mlp_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.pskel_mlp_destroy.argtypes = [C.c_void_p]
    L.pskel_set_cost_model.argtypes = [C.c_void_p]


_setup()


def sched_tuple(s: P.Schedule):
    return (s.tile_w, s.tile_h, s.tile_d, s.time_steps, s.ctas)


def candidates(st: P.Stencil, W: int, H: int, iterations: int):
    n = P.lib.pskel_candidates2d(C.byref(st), W, H, iterations, None, 0)
    arr = (P.Schedule * max(n, 1))()
    P.lib.pskel_candidates2d(C.byref(st), W, H, iterations, arr, n)
    return [arr[i] for i in range(n)]


def time_schedules(st: P.Stencil, a, b, iterations: int, scheds, reps: int = 3, pitch: int = 0, width=None,
                   height=None, stream=None):
    """Median ms of each schedule on device buffers a, b (overwritten)."""
    H = height if height is not None else a.shape[0]
    W = width if width is not None else a.shape[1]
    arr = (P.Schedule * len(scheds))(*scheds)
    ms = (C.c_double * len(scheds))()
    P._check(P.lib.pskel_time2d(C.byref(st), P._ptr(a), P._ptr(b), W, H, pitch, iterations, arr, len(scheds), reps,
                                ms, stream))
    return np.array(ms[:], dtype=np.float64)


def time_in_batch(st: P.Stencil, pool, W: int, H: int, iterations: int, scheds, reps: int = 3, stream=None):
    """Median ms per grid of each schedule inside a batched launch of copies of
    the grid (buffers from the device tensor `pool`, overwritten)."""
    arr = (P.Schedule * len(scheds))(*scheds)
    ms = (C.c_double * len(scheds))()
    cp = (C.c_int32 * len(scheds))()
    nbytes = pool.numel() * pool.element_size()
    P._check(P.lib.pskel_time_batch2d(C.byref(st), P._ptr(pool), nbytes, W, H, iterations, arr, len(scheds), reps,
                                      ms, cp, stream))
    return np.array(ms[:], dtype=np.float64), np.array(cp[:], dtype=np.int64)


def exhaustive(st: P.Stencil, a, b, iterations: int, reps: int = 3, pitch: int = 0, width=None, height=None):
    """(best schedule, its ms, all candidates, their ms)."""
    H = height if height is not None else a.shape[0]
    W = width if width is not None else a.shape[1]
    cands = candidates(st, W, H, iterations)
    ms = time_schedules(st, a, b, iterations, cands, reps=reps, pitch=pitch, width=W, height=H)
    i = int(np.argmin(ms))
    return cands[i], float(ms[i]), cands, ms


def ga_schedule(st: P.Stencil, W: int, H: int, iterations: int, seed: int = 1, popsize: int = 100, ngen: int = 2500):
    out = P.Schedule()
    score = C.c_double()
    P._check(P.lib.pskel_ga_schedule2d(C.byref(st), W, H, iterations, seed, popsize, ngen, C.byref(out),
                                       C.byref(score)))
    return out, score.value


def features(st: P.Stencil, W: int, H: int, iterations: int, s: P.Schedule) -> np.ndarray:
    f = (C.c_float * NFEAT)()
    P.lib.pskel_schedule_features2d(C.byref(st), W, H, iterations, C.byref(s), f)
    return np.array(f[:], dtype=np.float32)


def auto_schedule(st: P.Stencil, W: int, H: int, iterations: int) -> P.Schedule:
    out = P.Schedule()
    P._check(P.lib.pskel_auto_schedule2d(C.byref(st), W, H, iterations, C.byref(out)))
    return out


class CostModel:
    """The MLP cost model: predicts log(ms) of a (grid, schedule)."""

    def __init__(self, hidden: int = 64, layers: int = 3, seed: int = 1, in_dim: int = NFEAT, handle=None):
        self.h = C.c_void_p()
        if handle is not None:
            self.h = handle
        else:
            P._check(P.lib.pskel_mlp_create(in_dim, hidden, layers, seed, C.byref(self.h)))
        self.in_dim = in_dim

    @classmethod
    def load(cls, path: str) -> "CostModel":
        h = C.c_void_p()
        P._check(P.lib.pskel_mlp_load(str(path).encode(), C.byref(h)))
        return cls(handle=h)

    def save(self, path: str):
        P._check(P.lib.pskel_mlp_save(self.h, str(path).encode()))

    @property
    def num_params(self) -> int:
        return P.lib.pskel_mlp_num_params(self.h)

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, dtype=np.float32)
        P._check(P.lib.pskel_mlp_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        P._check(P.lib.pskel_mlp_set_params(self.h, p.ctypes.data))

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.zeros(X.shape[0], dtype=np.float32)
        P._check(P.lib.pskel_mlp_predict(self.h, X.ctypes.data, X.shape[0], y.ctypes.data))
        return y

    def gradient(self, X: np.ndarray, y: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_float()
        P._check(P.lib.pskel_mlp_gradient(self.h, X.ctypes.data, y.ctypes.data, X.shape[0], g.ctypes.data,
                                          C.byref(loss)))
        return g, loss.value

    def train(self, X: np.ndarray, y: np.ndarray, epochs: int = 2000, lr: float = 3e-3) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_float()
        P._check(P.lib.pskel_mlp_train(self.h, X.ctypes.data, y.ctypes.data, X.shape[0], epochs, lr, C.byref(loss)))
        return loss.value

    def pick(self, st: P.Stencil, W: int, H: int, iterations: int) -> P.Schedule:
        cands = candidates(st, W, H, iterations)
        X = np.stack([features(st, W, H, iterations, c) for c in cands])
        return cands[int(np.argmin(self.predict(X)))]

    def register(self):
        """Make this model the one runIterativeAutoGPU / pskel_auto_schedule2d uses."""
        P._check(P.lib.pskel_set_cost_model(self.h))

    def close(self):
        if self.h:
            P.lib.pskel_set_cost_model(None)
            P.lib.pskel_mlp_destroy(self.h)
            self.h = C.c_void_p()

