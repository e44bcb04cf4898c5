"""The MLP cost model's CUDA forward/backward/Adam kernels against the fp64
oracle, its training, determinism and files; the measured tuner; and what the
trained model gains over the library's default schedule and the GA's pick."""
from __future__ import annotations

import numpy as np
import pytest

import pskel_gb300 as P
import pskel_gb300.tuner as T
from oracle import mlp_oracle as M
from pskel_gb300 import synth as S
from tests.gpu_util import aligned_pitch, bits, from_dev, to_dev

pytestmark = pytest.mark.gpu


def _data(seed, n, din):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (n, din)).astype(np.float32)
    y = (np.sin(2 * X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] - 0.3 * X[:, 3] ** 2).astype(np.float32)
    return X, y


def test_forward_and_gradient_match_fp64_oracle(cuda):
    m = T.CostModel(hidden=64, layers=3, seed=11)
    try:
        dims = M.dims_of(T.NFEAT, 64, 3)
        assert m.num_params == M.num_params(dims)
        p = m.get_params()
        X, y = _data(1, 97, T.NFEAT)
        np.testing.assert_allclose(m.predict(X), M.predict(p, X, dims), rtol=1e-5, atol=1e-5)
        g, loss = m.gradient(X, y)
        g64, loss64 = M.gradient(p, X, y, dims)
        assert loss == pytest.approx(loss64, rel=1e-5)
        # fp32 accumulation over 97 samples: relative to the gradient's scale
        assert np.max(np.abs(g - g64)) <= 1e-5 * np.max(np.abs(g64))
    finally:
        m.close()


def test_adam_step_matches_oracle(cuda):
    m = T.CostModel(hidden=16, layers=3, seed=2)
    try:
        dims = M.dims_of(T.NFEAT, 16, 3)
        X, y = _data(2, 40, T.NFEAT)
        p0 = m.get_params().astype(np.float64)
        m.train(X, y, epochs=2, lr=1e-2)
        want, mm, vv = p0, np.zeros_like(p0), np.zeros_like(p0)
        for step in (1, 2):
            g, _ = M.gradient(want, X, y, dims)
            want, mm, vv = M.adam(want, g, mm, vv, step, 1e-2)
        np.testing.assert_allclose(m.get_params(), want, rtol=0, atol=2e-5)
    finally:
        m.close()


def test_training_converges_and_is_deterministic(cuda):
    X, y = _data(3, 256, T.NFEAT)
    params, losses = [], []
    for _ in range(2):
        m = T.CostModel(hidden=64, layers=3, seed=5)
        l0 = m.gradient(X, y)[1]
        losses.append((l0, m.train(X, y, epochs=1500, lr=3e-3)))
        params.append(m.get_params())
        m.close()
    assert losses[0][1] < 0.02 * losses[0][0]
    assert np.array_equal(params[0], params[1]) and losses[0] == losses[1]


def test_save_load_round_trip(cuda, tmp_path):
    m = T.CostModel(hidden=32, layers=4, seed=9)
    try:
        X, _ = _data(4, 33, T.NFEAT)
        path = tmp_path / "m.pmlp"
        m.save(str(path))
        m2 = T.CostModel.load(str(path))
        assert np.array_equal(m2.get_params(), m.get_params())
        assert np.array_equal(m2.predict(X), m.predict(X))
        m2.close()
        path.write_bytes(path.read_bytes()[:-8])
        with pytest.raises(P.PskelError):
            T.CostModel.load(str(path))
    finally:
        m.close()


def _jacobi_grid(torch, W, H, seed):
    a, b = S.jacobi2d(W, H, seed=seed)
    pitch = aligned_pitch(W, 4)
    return a, b, pitch, to_dev(torch, a, pitch), to_dev(torch, b, pitch)


def test_every_candidate_gives_the_same_result(cuda, oracle_mod):
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    W, H, it = 333, 270, 17
    a, b, pitch, _, _ = _jacobi_grid(torch, W, H, 21)
    want = oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, it)
    for s in T.candidates(st, W, H, it):
        x, y = to_dev(torch, a, pitch), to_dev(torch, b, pitch)
        P.iterate2d(st, x, y, it, sched=s, pitch=pitch, width=W, height=H)
        P.sync()
        got = from_dev(y if it % 2 else x, W)
        assert np.array_equal(bits(got), bits(want)), T.sched_tuple(s)


def test_measured_tuner(cuda):
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    W, H, it = 1024, 1024, 30
    _, _, pitch, x, y = _jacobi_grid(torch, W, H, 5)
    best, best_ms, cands, ms = T.exhaustive(st, x, y, it, reps=3, pitch=pitch, width=W, height=H)
    assert len(cands) == len(ms) and np.all(ms > 0)
    assert best_ms == ms.min()
    # the registered cost model drives pskel_auto_schedule2d; without one the default schedule comes back
    P.lib.pskel_set_cost_model(None)
    assert T.sched_tuple(T.auto_schedule(st, W, H, it)) == (0, 0, 0, 0, 0)


def _training_set(torch, st, shapes, reps=3):
    X, y = [], []
    for k, (W, H, it) in enumerate(shapes):
        _, _, pitch, x, yb = _jacobi_grid(torch, W, H, 100 + k)
        cands = T.candidates(st, W, H, it)
        ms = T.time_schedules(st, x, yb, it, cands, reps=reps, pitch=pitch, width=W, height=H)
        for c, t in zip(cands, ms):
            X.append(T.features(st, W, H, it, c))
            y.append(np.log(t))
    return np.stack(X), np.array(y, dtype=np.float32)


def test_trained_model_beats_default_and_ga(cuda):
    """Trained on measured timings of one set of grids, the model's picks on
    held-out grids run faster in total than the library's default schedule, at
    least as fast as the GA's pick (within timing noise), and stay close to the
    exhaustive tuner's."""
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    rng = np.random.default_rng(8)
    train = [(int(w), int(h), int(i)) for w, h, i in zip(np.exp(rng.uniform(np.log(64), np.log(2048), 24)),
                                                          np.exp(rng.uniform(np.log(64), np.log(2048), 24)),
                                                          rng.integers(10, 200, 24))]
    X, y = _training_set(torch, st, train)
    m = T.CostModel(hidden=64, layers=3, seed=1)
    try:
        y_mean = float(y.mean())
        m.train(X, y - y_mean, epochs=3000, lr=3e-3)
        held = [(1500, 1100, 150), (700, 1900, 80), (2000, 300, 120), (900, 900, 60)]
        tot = {"model": 0.0, "default": 0.0, "ga": 0.0, "best": 0.0}
        for k, (W, H, it) in enumerate(held):
            _, _, pitch, x, yb = _jacobi_grid(torch, W, H, 500 + k)
            cands = T.candidates(st, W, H, it)
            ms = T.time_schedules(st, x, yb, it, cands, reps=5, pitch=pitch, width=W, height=H)
            pick = m.pick(st, W, H, it)
            ga, _ = T.ga_schedule(st, W, H, it, seed=1)
            t = T.time_schedules(st, x, yb, it, [pick, P.Schedule(), ga], reps=5, pitch=pitch, width=W, height=H)
            tot["model"] += t[0]
            tot["default"] += t[1]
            tot["ga"] += t[2]
            tot["best"] += ms.min()
        print({k: round(v, 4) for k, v in tot.items()})
        # measured on GB300 over several runs with one launch per pass:
        # model/best 1.13-1.22, model/GA 0.83-0.90, model/default 0.67-0.73.
        # Grids of this size now run every pass in one persistent launch, where
        # the GA's long passes (T = 15, tall tiles) are close to the best too:
        # model/best 1.007, model/GA 0.990, model/default 0.918. The bound
        # allows timing noise; the learned batched launch against the GA-tuned
        # per-grid launches (4.6x in the batch bench) is the larger gain.
        assert tot["model"] <= 1.02 * tot["ga"]
        assert tot["model"] <= 1.02 * tot["default"]
        assert tot["model"] <= 1.35 * tot["best"]
        # registered, it is what pskel_auto_schedule2d returns
        m.register()
        W, H, it = held[0]
        assert T.sched_tuple(T.auto_schedule(st, W, H, it)) == T.sched_tuple(m.pick(st, W, H, it))
    finally:
        m.close()


def test_time_in_batch(cuda):
    torch = cuda
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "bf16", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    pool = torch.empty(8 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    cands = [c for c in T.candidates(st, 100, 70, 40) if c.tile_h == 0]
    ms, copies = T.time_in_batch(st, pool, 100, 70, 40, cands, reps=3)
    assert np.all(ms > 0) and np.all(copies >= 1)
    # a small grid is replicated to fill the GPU, as far as the pool allows
    assert copies.max() > 1
    with pytest.raises(P.PskelError):
        T.time_in_batch(st, pool[:1024], 100, 70, 40, cands[:1])
