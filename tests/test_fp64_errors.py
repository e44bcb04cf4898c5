"""The FP64 errors the benchmark reports beside each float workload
(tests/golden/fp64_errors.json, written by tests/golden/make_fp64_errors.py):
every float workload has an entry, the Jacobi entry is recomputed here from
the oracle and must match exactly, and the bench line carries them."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

import bench
from tests.golden import make_fp64_errors as M

FIX = json.loads((Path(__file__).resolve().parent / "golden" / "fp64_errors.json").read_text())


def test_every_float_workload_has_an_entry():
    floats = [n for n, wl in bench.WORKLOADS.items() if n != "life"]
    assert sorted(floats) == sorted(M.FLOAT_WORKLOADS)
    for name in M.FLOAT_WORKLOADS:
        e = FIX[name]
        assert e["dtype"] == bench.WORKLOADS[name]["dtype"]
        for k in ("max_abs", "max_rel", "rel_l2"):
            assert e[k] >= 0.0
        # fp32 results stay close to FP64; bf16 storage loses bits every step
        if e["dtype"] == "f32":
            assert e["rel_l2"] < 1e-5 and e["max_rel"] < 1e-4
        else:
            assert e["rel_l2"] < 0.2


@pytest.mark.parametrize("name", ["jacobi", "jacobi_bf16"])
def test_entry_recomputed_from_the_oracle(name):
    got = M.make(name)
    want = FIX[name]
    for k in ("max_abs", "max_rel", "rel_l2", "input_sha", "iterations", "dtype"):
        assert got[k] == want[k], k


def test_bench_reports_them():
    for name in M.FLOAT_WORKLOADS:
        e = bench.fp64_error(dict(bench.WORKLOADS[name], name=name))
        assert e["max_abs"] == FIX[name]["max_abs"] and "source" in e
    assert bench.fp64_error(dict(bench.WORKLOADS["life"], name="life"))["kind"] == "integer"
