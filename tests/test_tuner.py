"""Schedule search host logic (no GPU): the fp64 MLP oracle against finite
differences, the candidate space, the features, and the genetic search against
a brute-force maximum of the reference's analytic objective."""
from __future__ import annotations

import math

import numpy as np
import pytest

import pskel_gb300 as P
import pskel_gb300.tuner as T
from oracle import mlp_oracle as M
from pskel_gb300 import synth as S


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    dims = M.dims_of(5, 7, 3)
    p = rng.normal(0, 0.5, M.num_params(dims))
    X = rng.normal(0, 1, (11, 5))
    y = rng.normal(0, 1, 11)
    g, loss = M.gradient(p, X, y, dims)
    assert loss == pytest.approx(M.loss(p, X, y, dims), rel=1e-12)
    num = np.zeros_like(p)
    h = 1e-6
    for i in range(p.size):
        e = np.zeros_like(p)
        e[i] = h
        num[i] = (M.loss(p + e, X, y, dims) - M.loss(p - e, X, y, dims)) / (2 * h)
    assert np.max(np.abs(g - num)) < 1e-7 * max(1.0, np.max(np.abs(num)))


def _jacobi(dtype="f32", keep=None):
    return P.make_stencil(P.OP_LINEAR, dtype, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)


def test_candidates_fast_path():
    keep = P._Keep()
    st = _jacobi(keep=keep)
    c = [T.sched_tuple(s) for s in T.candidates(st, 1024, 768, 100)]
    assert len(c) == 16 and len(set(c)) == 16
    assert all(s[3] % 2 == 1 and 1 <= s[3] <= 15 and s[1] in (0, 130) for s in c)
    # never more steps per pass than iterations
    assert {s.time_steps for s in T.candidates(st, 64, 64, 4)} == {1, 3}


def test_candidates_life_and_generic():
    keep = P._Keep()
    life = P.make_stencil(P.OP_LIFE, "u8", S.MOORE8_OFFSETS, keep=keep)
    c = [T.sched_tuple(s) for s in T.candidates(life, 512, 512, 1000)]
    assert c and all(s[3] % 2 == 1 for s in c)
    gen = P.make_stencil(P.OP_LINEAR, "f32", [(0, 0), (2, 0), (-2, 0), (0, 2), (0, -2)], [0.2] * 5, keep=keep)
    c = [T.sched_tuple(s) for s in T.candidates(gen, 512, 512, 1000)]
    assert {s[0] for s in c} == {64, 128} and {s[1] for s in c} == {32, 64}


def test_features():
    keep = P._Keep()
    st = _jacobi("bf16", keep=keep)
    s = P.Schedule(tile_h=130, time_steps=6)
    f = T.features(st, 2048, 512, 100, s)
    # even steps per pass round down to odd (5): 20 passes; tall tile 128 x 130
    # loaded, 112 x 120 core (x halo rounded up to 8 bf16 cells): 19 x 5 tiles
    red = 128 * 130 / (112 * 120)
    np.testing.assert_allclose(f, [11, 9, math.log2(100), 5 / 8, 1, 0.5, 0, math.log2(20), math.log2(red),
                                   math.log2(95), math.log2(2048 * 512 * 100 * red)], rtol=1e-6)


@pytest.mark.parametrize("W,H,iters,dtype", [(1024, 1024, 100, "f32"), (4096, 3000, 500, "bf16"),
                                             (300, 200, 10, "f32")])
def test_ga_reaches_the_objective_maximum(W, H, iters, dtype):
    keep = P._Keep()
    st = _jacobi(dtype, keep=keep)
    s, score = T.ga_schedule(st, W, H, iters, seed=7, popsize=100, ngen=600)
    esz = 2 if dtype == "bf16" else 4
    budget = 227 * 1024  # one CTA's opt-in shared memory on this part (no GPU here: the library's fallback)
    hmax = M.max_height(128, H, esz, budget)
    best = 0.0
    for h in np.linspace(1, hmax, 400):
        for it in np.linspace(1, iters, 400):
            best = max(best, M.objective2d(h, it, 128, H, iters, 1, esz, budget))
    assert score >= 0.97 * best
    assert score <= best * 1.02
    # deterministic for a seed
    s2, score2 = T.ga_schedule(st, W, H, iters, seed=7, popsize=100, ngen=600)
    assert T.sched_tuple(s) == T.sched_tuple(s2) and score == score2
    assert s.time_steps % 2 == 1 and 1 <= s.time_steps <= 15


def test_cost_model_file_errors(tmp_path):
    bad = tmp_path / "bad.pmlp"
    bad.write_bytes(b"not a model at all")
    with pytest.raises(P.PskelError):
        T.CostModel.load(str(bad))
    with pytest.raises(P.PskelError):
        T.CostModel.load(str(tmp_path / "missing.pmlp"))
