"""One PSkel application written only against the reference's API
(tests/cpp/user_app.cu: user stencilKernel functors, Stencil2D/3D, their run
methods), built unchanged against two header sets:

* the reference's own headers (the oracle's copy, oracle/_ref/src): with g++
  and PSKEL_OMP, run here, results bit for bit the oracle's; with nvcc and
  PSKEL_CUDA, compiled (its 2D GPU scenarios compile; there is no GPU here);
* this repository's include/: with nvcc for sm_103a, linked to the library;
  its GPU and host scenarios run on the GPU machine (marked gpu).

The reference's declarations: PSkelStencil.h:139-156 (the functor) and
247-306 (the run methods)."""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from pskel_gb300 import synth as S

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "user_app.cu"
REF = ROOT / "oracle" / "_ref"
BUILD = ROOT / "tests" / "cpp" / "_build"
NVCC = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-fmad=false"]


def ref_headers():
    if not (REF / "src" / "PSkelStencil.hpp").is_file():
        import oracle
        oracle.build_ref()
    if not (REF / "src" / "PSkelStencil.hpp").is_file():
        pytest.skip("the oracle's copy of the reference headers is not prepared")
    return ["-include", "cstring", "-I", str(REF / "shim"), "-I", str(REF / "src")]


def run(exe, scenario, a, b, iters):
    H, W = a.shape[0], a.shape[1]
    D = a.shape[2] if a.ndim == 3 else 1
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        a.tofile(d / "in")
        b.tofile(d / "out")
        r = subprocess.run([str(exe), scenario, str(W), str(H), str(D), str(iters), str(d / "in"), str(d / "out"),
                            str(d / "res")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return np.fromfile(d / "res", dtype=a.dtype).reshape(a.shape)


def cases(oracle_mod, scenario, iters):
    if scenario.startswith("jacobi"):
        a, b = S.jacobi2d(131, 97, seed=iters)
        b = b.copy()
        b[0, :] = 0.5
        return a, b, oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
    if scenario.startswith("life"):
        a, _ = S.life(133, 91, seed=iters)
        b = S.bernoulli_u8(iters + 9, S.S_GRID, a.shape, 0.5)
        return a, b, oracle_mod.life(a, b, iters)
    a, _ = S.heat3d(23, 19, 40, seed=iters)
    b = S.uniform_f32(iters + 3, S.S_GRID, a.shape)
    want, _ = oracle_mod.lin3d(a, b, S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters, halo=0.5)
    return a, b, want


@pytest.fixture(scope="module")
def ref_host_app(tmp_path_factory):
    exe = tmp_path_factory.mktemp("user_app") / "user_app_ref"
    subprocess.run(["g++", "-x", "c++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-DPSKEL_OMP",
                    *ref_headers(), "-w", str(SRC), "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("scenario", ["jacobi_cpu", "life_cpu", "heat_cpu"])
@pytest.mark.parametrize("iters", [1, 4, 7])
def test_user_app_on_reference_headers(ref_host_app, oracle_mod, scenario, iters):
    a, b, want = cases(oracle_mod, scenario, iters)
    got = run(ref_host_app, scenario, a, b, iters)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))


def test_user_app_gpu_build_compiles_on_reference_headers(tmp_path):
    """The reference's 2D GPU path (PSKEL_CUDA) compiles with the same source."""
    subprocess.run([*NVCC, "-DPSKEL_CUDA", "-DPSKEL_OMP", "-Xcompiler", "-fopenmp", *ref_headers(), "-w", "-c",
                    str(SRC), "-o", str(tmp_path / "user_app_ref.o")], check=True)


def build_ours():
    BUILD.mkdir(exist_ok=True)
    exe = BUILD / "user_app"
    lib_dir = ROOT / "pskel_gb300"
    if not exe.exists() or exe.stat().st_mtime < max(SRC.stat().st_mtime,
                                                      *(p.stat().st_mtime for p in (ROOT / "include").glob("*.h"))):
        subprocess.run([*NVCC, "-DPSKEL_CUDA", "-DPSKEL_OMP", "-Xcompiler", "-fopenmp,-ffp-contract=off",
                        f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe), f"-L{lib_dir}", "-lpskel_gb300",
                        f"-Xlinker=-rpath,{lib_dir}", "-lgomp"], check=True, capture_output=True)
    return exe


def test_user_app_builds_on_our_headers():
    if not (ROOT / "pskel_gb300" / "libpskel_gb300.so").exists():
        pytest.skip("library not built")
    assert build_ours().exists()


@pytest.mark.gpu
@pytest.mark.parametrize("scenario", ["jacobi_gpu", "jacobi_cpu", "life_gpu", "life_cpu", "heat_cpu"])
@pytest.mark.parametrize("iters", [1, 4, 7])
def test_user_app_on_our_headers(cuda, oracle_mod, scenario, iters):
    a, b, want = cases(oracle_mod, scenario, iters)
    got = run(build_ours(), scenario, a, b, iters)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
