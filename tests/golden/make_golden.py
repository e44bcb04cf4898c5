"""Generate the golden fixtures from the reference's own runIterativeCPU.

Runs ``oracle/_ref/pskel_ref`` (the reference headers compiled by
``oracle/make_ref.py``) on small seeded inputs and stores its outputs in
``tests/golden/golden.npz``. The inputs are regenerated from their seeds by
``pskel_gb300.synth``; their sha256 is stored next to the outputs so a change
of the generator is detected instead of silently invalidating the fixtures.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from pskel_gb300 import synth as S  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"

# A 9-entry radius-2 mask with weights that are not exact in binary, so the
# summation order is exercised.
STAR9_OFFSETS = [(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1), (-2, 0), (2, 0), (0, -2), (0, 2)]
STAR9_WEIGHTS = [0.2, 0.15, 0.1, 0.15, 0.1, 0.075, 0.05, 0.1, 0.07]


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cases():
    """(name, kind, params) for every fixture; params regenerate the inputs."""
    out = []
    for it in (1, 2, 7):
        out.append((f"lin2d_f32_jacobi_it{it}", "lin2d", dict(W=37, H=29, seed=3, iters=it, dtype="f32", mask="jacobi")))
    out.append(("lin2d_f32_star9_it5", "lin2d", dict(W=41, H=35, seed=4, iters=5, dtype="f32", mask="star9")))
    out.append(("lin2d_f64_jacobi_it7", "lin2d", dict(W=37, H=29, seed=3, iters=7, dtype="f64", mask="jacobi")))
    out.append(("lin2d_bf16_jacobi_it7", "lin2d", dict(W=37, H=29, seed=3, iters=7, dtype="bf16", mask="jacobi")))
    for it in (1, 2, 13):
        out.append((f"life_it{it}", "life", dict(W=67, H=45, seed=5, iters=it)))
    for dt in ("f32", "f64", "bf16"):
        out.append((f"advect_{dt}_it9", "advect", dict(W=40, H=33, seed=2, iters=9, dtype=dt)))
    for dt in ("f32", "f64", "bf16"):
        out.append((f"lin3d_{dt}_it7", "lin3d", dict(W=11, H=9, D=13, seed=4, iters=7, dtype=dt, halo=0.5, every=3)))
    return out


def _cast(x, dtype):
    if dtype == "f64":
        return x.astype(np.float64)
    if dtype == "bf16":
        return S.f32_to_bf16(x)
    return x


def inputs(kind, p):
    """Regenerate the inputs of a fixture; returns a dict of arrays."""
    if kind == "lin2d":
        a, b = S.jacobi2d(p["W"], p["H"], seed=p["seed"])
        # give the output array its own ring so the ring semantics are visible
        b = b.copy()
        b[0, :] = 0.5
        b[:, -1] = 0.25
        return {"in": _cast(a, p["dtype"]), "out": _cast(b, p["dtype"])}
    if kind == "life":
        a, _ = S.life(p["W"], p["H"], seed=p["seed"])
        b = S.bernoulli_u8(p["seed"] + 100, S.S_GRID, a.shape, 0.5)
        return {"in": a, "out": b}
    if kind == "advect":
        a, b, u, v = S.advect2d(p["W"], p["H"], seed=p["seed"])
        dt = p["dtype"]
        return {"in": _cast(a, dt), "out": _cast(b, dt), "u": _cast(u, dt), "v": _cast(v, dt)}
    if kind == "lin3d":
        a, _ = S.heat3d(p["W"], p["H"], p["D"], seed=p["seed"])
        b = S.uniform_f32(p["seed"] + 100, S.S_GRID, a.shape)
        return {"in": _cast(a, p["dtype"]), "out": _cast(b, p["dtype"])}
    raise ValueError(kind)


def mask_of(p):
    if p.get("mask") == "star9":
        return STAR9_OFFSETS, STAR9_WEIGHTS
    return S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS


def run_reference(kind, p, x):
    if kind == "lin2d":
        off, wt = mask_of(p)
        return {"result": oracle.ref_lin2d(x["in"], x["out"], off, wt, p["iters"], dtype=p["dtype"])}
    if kind == "life":
        res, _ = oracle.ref_life(x["in"], x["out"], p["iters"])
        return {"result": res}
    if kind == "advect":
        return {"result": oracle.ref_advect(x["in"], x["out"], x["u"], x["v"], p["iters"], S.ADVECT_K, S.ADVECT_DT,
                                            S.ADVECT_INV_DX, dtype=p["dtype"])}
    if kind == "lin3d":
        res, norms = oracle.ref_lin3d(x["in"], x["out"], S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, p["iters"],
                                      halo=p["halo"], dtype=p["dtype"], every=p["every"])
        return {"result": res, "norms": norms}
    raise ValueError(kind)


def main():
    if not oracle.have_ref():
        oracle.build_ref()
    if not oracle.have_ref():
        raise SystemExit("oracle/_ref/pskel_ref is not built (needs the reference headers)")
    store = {}
    for name, kind, p in cases():
        x = inputs(kind, p)
        store[f"{name}/input_sha"] = np.array(sha(*[x[k] for k in sorted(x)]))
        for k, v in run_reference(kind, p, x).items():
            store[f"{name}/{k}"] = v
    np.savez_compressed(OUT, **store)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(cases())} cases)")


if __name__ == "__main__":
    main()
