"""The reference's own GPU path (``Stencil2D::runIterativeGPU``: one
``stencilTilingCU`` launch per step with a device synchronisation after each,
PSkelStencil.hpp:1046-1097, :572-652, :1764-1792), compiled from its headers
by ``oracle/make_ref.py`` into ``oracle/_ref/pskel_ref_gpu`` and run beside the
library as the plain-GPU comparator.

Its ring is not the CPU path's: the output array is never copied to the
device (PSkelStencil.hpp:1071), so from the second step on the ring read is
whatever the fresh device allocation holds, and the difference moves inward
one cell per step. Cells farther than ``iters`` from the edge agree with the
reference's CPU path (the oracle) bit for bit on the Game of Life, and on the
Jacobi mask (weights 0.25: a contracted multiply-add rounds like the separate
product and sum); the first step agrees everywhere inside the ring. The
timings are printed as ``REF-GPU`` lines."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from pskel_gb300 import synth as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_gpu(cuda):
    if not oracle.have_ref_gpu():
        oracle.build_ref()
    if not oracle.have_ref_gpu():
        pytest.skip("oracle/_ref/pskel_ref_gpu is not built (needs the reference headers and nvcc)")
    return oracle


def core(x, m):
    return x[m:-m, m:-m]


@pytest.mark.parametrize("W,H,iters", [(1000, 777, 7), (1024, 1024, 8), (131, 67, 1), (131, 67, 2)])
def test_reference_gpu_life_matches_oracle_away_from_ring(ref_gpu, oracle_mod, W, H, iters):
    a, b = S.life(W, H, seed=iters)
    got, t = ref_gpu.ref_gpu_life(a, b, iters)
    want = oracle_mod.life(a, b, iters)
    assert np.array_equal(core(got, iters), core(want, iters))
    print("REF-GPU life", W, H, iters, t)


@pytest.mark.parametrize("W,H,iters", [(300, 200, 5), (1024, 1024, 6)])
def test_reference_gpu_jacobi_matches_oracle_away_from_ring(ref_gpu, oracle_mod, W, H, iters):
    a, b = S.jacobi2d(W, H, seed=iters)
    got, t = ref_gpu.ref_gpu_lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
    want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters)
    assert np.array_equal(core(got, iters).view(np.uint32), core(want, iters).view(np.uint32))
    print("REF-GPU jacobi", W, H, iters, t)
