"""The C++ drop-in API (include/PSkel*.h) on the GPU.

tests/cpp/dropin_app.cu is a PSkel application written against the
reference's API (Stencil2D/3D, Array2D/3D, Mask2D/3D, user stencilKernel
functors). It is compiled here with nvcc against the drop-in headers and
libpskel_gb300.so, run on seeded inputs, and its results are compared bit for
bit with the oracle: library paths (tagged Args), user-functor paths (kernels
generated from the functor, compiled with -fmad=false so the functor's sums
are not contracted, as in the oracle), the schedule-taking overloads, the
host runIterativeCPU, and the Map skeleton (include/PSkelMap.h). Host code is
compiled with -ffp-contract=off: gcc on aarch64 contracts a*b+c into one
fused multiply-add by default, which the oracle does not do.
"""
from __future__ import annotations

import json
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from pskel_gb300 import synth as S
from tests.gpu_util import bits

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
APP_SRC = ROOT / "tests" / "cpp" / "dropin_app.cu"
BUILD = ROOT / "tests" / "cpp" / "_build"
APP = BUILD / "dropin_app"


@pytest.fixture(scope="module")
def app():
    BUILD.mkdir(exist_ok=True)
    lib_dir = ROOT / "pskel_gb300"
    if not APP.exists() or APP.stat().st_mtime < max(APP_SRC.stat().st_mtime,
                                                      *(p.stat().st_mtime for p in (ROOT / "include").glob("*.h"))):
        cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-fmad=false",
               "-Xcompiler", "-fopenmp,-ffp-contract=off", "-DPSKEL_OMP", f"-I{ROOT / 'include'}", str(APP_SRC), "-o", str(APP),
               f"-L{lib_dir}", "-lpskel_gb300", f"-Xlinker=-rpath,{lib_dir}", "-lgomp"]
        subprocess.run(cmd, check=True, capture_output=True)
    return APP


def run_app(app, scenario, a, b, iters, want_res=False, env=None, stdout=None):
    shape = a.shape
    H, W = shape[0], shape[1]
    D = shape[2] if len(shape) == 3 else 1
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        np.ascontiguousarray(a).tofile(d / "in")
        np.ascontiguousarray(b).tofile(d / "out")
        args = [str(app), scenario, str(W), str(H), str(D), str(iters), str(d / "in"), str(d / "out"),
                str(d / "res")]
        if want_res:
            args.append(str(d / "norms"))
        r = subprocess.run(args, capture_output=True, text=True, env=env)
        assert r.returncode == 0, r.stderr
        if stdout is not None:
            stdout.append(r.stdout)
        res = np.fromfile(d / "res", dtype=a.dtype).reshape(shape)
        norms = np.fromfile(d / "norms", dtype=np.float64) if want_res else None
        return res, norms


def jac(W, H, seed):
    a, b = S.jacobi2d(W, H, seed=seed)
    b = b.copy()
    b[0, :] = 0.5
    b[:, -1] = 0.25
    return a, b


@pytest.mark.parametrize("scenario", ["jacobi_lib", "jacobi_pyramid", "jacobi_tiling", "jacobi_auto", "jacobi_user",
                                      "jacobi_cpu"])
@pytest.mark.parametrize("iters", [1, 6, 13])
def test_dropin_jacobi(app, oracle_mod, scenario, iters):
    a, b = jac(203, 157, iters)
    got, _ = run_app(app, scenario, a, b, iters)
    want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("scenario", ["life_lib", "life_user"])
@pytest.mark.parametrize("iters", [1, 8, 31])
def test_dropin_life(app, oracle_mod, scenario, iters):
    a, _ = S.life(301, 227, seed=iters)
    b = S.bernoulli_u8(iters + 7, S.S_GRID, a.shape, 0.5)
    got, _ = run_app(app, scenario, a, b, iters)
    assert np.array_equal(got, oracle_mod.life(a, b, iters))


@pytest.mark.parametrize("scenario", ["heat_lib", "heat_user"])
@pytest.mark.parametrize("iters", [1, 4, 7])
def test_dropin_heat3d(app, oracle_mod, scenario, iters):
    a, _ = S.heat3d(37, 29, 48, seed=iters)
    b = S.uniform_f32(iters + 3, S.S_GRID, a.shape)
    got, norms = run_app(app, scenario, a, b, iters, want_res=(scenario == "heat_lib"))
    want, wnorms = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=0.5, every=2)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    if norms is not None:
        np.testing.assert_allclose(norms, wnorms, rtol=1e-12, atol=0)


def test_dropin_auto_with_cost_model(app, oracle_mod, tmp_path):
    """runIterativeAutoGPU with a cost-model file named by PSKEL_COST_MODEL:
    the model picks the schedule, the results stay the reference's."""
    import os

    import pskel_gb300.tuner as T
    m = T.CostModel(hidden=64, layers=3, seed=3)
    path = tmp_path / "model.pmlp"
    m.save(str(path))
    m.close()
    env = dict(os.environ, PSKEL_COST_MODEL=str(path))
    for iters in (7, 40):
        a, b = jac(517, 389, iters)
        got, _ = run_app(app, "jacobi_auto", a, b, iters, env=env)
        want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def affine(x, iters):
    # the app's mapKernel: out = 0.75 * in + 0.125, fp32 product then sum
    a, b = np.float32(0.75), np.float32(0.125)
    for _ in range(iters):
        x = (a * x).astype(np.float32) + b
    return x.astype(np.float32)


@pytest.mark.parametrize("scenario", ["map1d_gpu", "map1d_seq", "map2d_gpu", "map2d_cpu", "map3d_gpu"])
@pytest.mark.parametrize("iters", [1, 2, 5])
def test_dropin_map(app, scenario, iters):
    rng = np.random.default_rng(iters)
    shape = (17, 33, 9) if scenario.startswith("map3d") else (61, 130)
    a = rng.uniform(0, 1, shape).astype(np.float32)
    b = rng.uniform(0, 1, shape).astype(np.float32)
    a0 = a.copy()
    got, _ = run_app(app, scenario, a, b, iters)
    assert np.array_equal(got.view(np.uint32), affine(a0, iters).view(np.uint32))


@pytest.mark.parametrize("scenario,shape,budget", [
    ("jacobi_tiling", (157, 203), 200_000),   # slabs of tilingHeight = 32 rows, 5 steps per visit
    ("jacobi_auto", (700, 520), 2 << 20),     # slabs sized from the budget
    ("life_tiling", (227, 301), 100_000),
    ("heat_tiling", (29, 37, 48), 300_000),   # slabs of 8 h-planes, 3 steps per visit
    ("jacobi_user_tiling", (157, 203), 200_000),  # a user functor: slabs of 24 rows, 5 steps per visit
    ("jacobi_user_auto", (700, 520), 2 << 20),    # a user functor, slabs sized from the budget
    ("heat_user_tiling", (29, 37, 48), 300_000),  # a 3D user functor: slabs of 6 h-planes, 3 steps per visit
])
@pytest.mark.parametrize("iters", [1, 6, 13])
def test_dropin_out_of_core(app, oracle_mod, scenario, shape, budget, iters):
    """runIterativeTilingGPU / runIterativeAutoGPU on arrays larger than the
    device memory the application may use (PSKEL_DEVICE_BYTES caps it) run out
    of core, with the reference's results."""
    import os
    env = dict(os.environ, PSKEL_DEVICE_BYTES=str(budget))
    if scenario.startswith("life"):
        a, _ = S.life(shape[1], shape[0], seed=iters)
        b = S.bernoulli_u8(iters + 7, S.S_GRID, a.shape, 0.5)
        want = oracle_mod.life(a, b, iters)
    elif scenario.startswith("heat"):
        a, _ = S.heat3d(shape[1], shape[0], shape[2], seed=iters)
        b = S.uniform_f32(iters + 3, S.S_GRID, a.shape)
        want, _ = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=0.5)
    else:
        a, b = jac(shape[1], shape[0], iters)
        want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
    assert 2 * a.nbytes > budget
    out = []
    got, _ = run_app(app, scenario, a, b, iters, env=env, stdout=out)
    assert "out of core" in out[0]
    assert np.array_equal(bits(got), bits(want))


def smooth1d(x, iters):
    """The app's 1D stencil: sum_n w_n * in(i + o_n) in mask order, fp32,
    the halo value 0.5 outside the array (Mask::get, PSkelMask.hpp:387-395)."""
    off = [-2, -1, 0, 1, 3]
    wt = [np.float32(v) for v in (0.125, 0.25, 0.3, 0.2, 0.125)]
    x = x.astype(np.float32)
    W = x.size
    for _ in range(iters):
        pad = np.full(W + 5, np.float32(0.5), dtype=np.float32)
        pad[2:2 + W] = x
        acc = None
        for o, w in zip(off, wt):
            term = (w * pad[2 + o:2 + o + W]).astype(np.float32)
            acc = term if acc is None else (acc + term).astype(np.float32)
        x = acc
    return x


@pytest.mark.parametrize("scenario", ["stencil1d_gpu", "stencil1d_cpu"])
@pytest.mark.parametrize("W,iters", [(1, 1), (7, 2), (1000, 5), (100_003, 12)])
def test_dropin_stencil1d(app, scenario, W, iters):
    rng = np.random.default_rng(W + iters)
    a = rng.uniform(0, 1, (1, W)).astype(np.float32)
    b = rng.uniform(0, 1, (1, W)).astype(np.float32)
    got, _ = run_app(app, scenario, a, b, iters)
    want = smooth1d(a[0], iters)
    assert np.array_equal(got[0].view(np.uint32), want.view(np.uint32))


def coef_run(a, b, iters):
    """The app's Args2D functor restated: interior cells (ring 1) of the
    destination get c + k * (((n + s) + (w + e)) - 4c) in fp32, rounded per
    operation; each array keeps its ring; the result is in the output array
    for odd counts, in the input array for even ones."""
    H, W = a.shape
    hh, ww = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    k = (np.float32(0.05) + np.float32(0.2) * ((hh * 7 + ww * 3) % 11).astype(np.float32) / np.float32(10.0))
    k = k.astype(np.float32)
    x, y = a.astype(np.float32).copy(), b.astype(np.float32).copy()
    for it in range(iters):
        src, dst = (x, y) if it % 2 == 0 else (y, x)
        c = src[1:-1, 1:-1]
        s1 = (src[:-2, 1:-1] + src[2:, 1:-1]).astype(np.float32)
        s2 = (src[1:-1, :-2] + src[1:-1, 2:]).astype(np.float32)
        sm = (s1 + s2).astype(np.float32)
        d = (sm - (np.float32(4.0) * c).astype(np.float32)).astype(np.float32)
        dst[1:-1, 1:-1] = (c + (k[1:-1, 1:-1] * d).astype(np.float32)).astype(np.float32)
    return y if iters % 2 == 1 else x


@pytest.mark.parametrize("scenario", ["coef_gpu", "coef_cpu"])
@pytest.mark.parametrize("iters", [1, 4, 9])
def test_dropin_args_field(app, scenario, iters):
    """A user functor reading an Args2D field (mapped pinned host memory, the
    reference's Args, PSkelArgs.hpp) on the GPU and on the host."""
    rng = np.random.default_rng(iters)
    a = rng.uniform(0, 1, (97, 131)).astype(np.float32)
    b = rng.uniform(0, 1, (97, 131)).astype(np.float32)
    got, _ = run_app(app, scenario, a, b, iters)
    assert np.array_equal(got.view(np.uint32), coef_run(a, b, iters).view(np.uint32))


@pytest.mark.parametrize("iters", [1, 4, 9])
def test_dropin_args_field_out_of_core(app, iters):
    """The same functor out of core (slabs of 16 rows, 3 steps per visit):
    it must see grid coordinates, so the field is read at the right cells."""
    import os
    rng = np.random.default_rng(iters + 50)
    a = rng.uniform(0, 1, (97, 131)).astype(np.float32)
    b = rng.uniform(0, 1, (97, 131)).astype(np.float32)
    env = dict(os.environ, PSKEL_DEVICE_BYTES="60000")
    assert 2 * a.nbytes > 60000
    out = []
    got, _ = run_app(app, "coef_tiling", a, b, iters, env=env, stdout=out)
    assert "out of core" in out[0]
    assert np.array_equal(got.view(np.uint32), coef_run(a, b, iters).view(np.uint32))


@pytest.mark.parametrize("scenario", ["map1d_time", "stencil1d_time"])
def test_dropin_functor_throughput(app, scenario):
    """The grid-stride user-functor kernels (the Map skeleton and the 1D
    stencil) measured through the public API on 2^27 cells: one iteration's
    device time is the difference of two runs of different lengths divided by
    the difference of their iteration counts. A floor only (the kernels read
    and write each cell once per iteration, one cell per thread)."""
    r = subprocess.run([str(app), scenario, str(1 << 27), "1", "1", "1000", "-", "-", "-"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["iterations"] == [10, 1000] and line["GBps"] > 500, line


def test_dropin_args_field_throughput(app):
    """The Args2D functor (a per-cell coefficient read from mapped pinned host
    memory) measured through the public API on 8192 x 4096 cells: it is bound
    by the host link (4 bytes per cell and iteration over it). A floor only."""
    r = subprocess.run([str(app), "coef_time", "8192", "4096", "1", "110", "-", "-", "-"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["iterations"] == [11, 110] and line["host_link_GBps"] > 20, line
