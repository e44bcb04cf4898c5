"""The oracle (C restatement) against the reference's own runIterativeCPU.

``tests/golden/golden.npz`` holds outputs of the reference built from its own
headers (tests/golden/make_golden.py). Every oracle function must reproduce
them bit for bit. When the reference runner is built locally it is also
compared directly on further random cases.
"""
from __future__ import annotations

import numpy as np
import pytest

from pskel_gb300 import synth as S
from tests.golden import make_golden as G


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def _oracle(oracle, kind, p, x):
    if kind == "lin2d":
        off, wt = G.mask_of(p)
        return {"result": oracle.lin2d(x["in"], x["out"], off, wt, p["iters"], dtype=p["dtype"])}
    if kind == "life":
        return {"result": oracle.life(x["in"], x["out"], p["iters"])}
    if kind == "advect":
        return {"result": oracle.advect(x["in"], x["out"], x["u"], x["v"], p["iters"], S.ADVECT_K, S.ADVECT_DT,
                                        S.ADVECT_INV_DX, dtype=p["dtype"])}
    if kind == "lin3d":
        res, norms = oracle.lin3d(x["in"], x["out"], S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, p["iters"], halo=p["halo"],
                                  dtype=p["dtype"], every=p["every"])
        return {"result": res, "norms": norms}
    raise ValueError(kind)


@pytest.mark.parametrize("name,kind,p", G.cases(), ids=[c[0] for c in G.cases()])
def test_oracle_matches_reference_golden(oracle_mod, golden, name, kind, p):
    x = G.inputs(kind, p)
    assert str(golden[f"{name}/input_sha"]) == G.sha(*[x[k] for k in sorted(x)]), "input generator drifted"
    got = _oracle(oracle_mod, kind, p, x)
    for k, v in got.items():
        ref = golden[f"{name}/{k}"]
        assert v.shape == ref.shape
        assert np.array_equal(_bits(v), _bits(ref)), f"{name}/{k} differs from the reference"


def test_golden_ring_semantics(golden):
    # even iteration counts return the input array's ring, odd ones the output's
    x = G.inputs("lin2d", dict(W=37, H=29, seed=3, dtype="f32"))
    odd = golden["lin2d_f32_jacobi_it7/result"]
    even = golden["lin2d_f32_jacobi_it2/result"]
    assert np.array_equal(odd[0, :], x["out"][0, :])
    assert np.array_equal(even[0, :], x["in"][0, :])


@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_vs_reference_random(oracle_mod, seed):
    if not oracle_mod.have_ref():
        pytest.skip("reference runner not built here")
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(5, 60)), int(rng.integers(5, 60))
    a = S.uniform_f32(seed, 1, (H, W))
    b = S.uniform_f32(seed, 2, (H, W))
    off = [(int(rng.integers(-2, 3)), int(rng.integers(-2, 3))) for _ in range(6)]
    wt = [float(x) for x in rng.random(6).astype(np.float32)]
    it = int(rng.integers(0, 6))
    r1 = oracle_mod.lin2d(a, b, off, wt, it)
    r2 = oracle_mod.ref_lin2d(a, b, off, wt, it)
    assert np.array_equal(_bits(r1), _bits(r2))
    L0 = S.bernoulli_u8(seed, 3, (H, W), 0.4)
    L1 = S.bernoulli_u8(seed, 4, (H, W), 0.4)
    r1 = oracle_mod.life(L0, L1, it + 3)
    r2, _ = oracle_mod.ref_life(L0, L1, it + 3)
    assert np.array_equal(r1, r2)


def test_bf16_rounding_matches_oracle(oracle_mod):
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5e-3, 3.4e38, np.inf, -np.inf, 0.0, -0.0, 1e-40],
                 dtype=np.float32)
    ours = S.f32_to_bf16(x)
    lib = oracle_mod.lib()
    import ctypes as C
    lib.oracle_f32_to_bf16.restype = C.c_uint16
    theirs = np.array([lib.oracle_f32_to_bf16(C.c_float(float(v))) for v in x], dtype=np.uint16)
    assert np.array_equal(ours, theirs)
