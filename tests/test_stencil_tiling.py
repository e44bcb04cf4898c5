"""StencilTiling::tile (the drop-in's include/PSkelStencilTiling.h) against the
reference's own (PSkelStencilTiling.h:85-148, from the oracle's copy of the
reference headers): the same driver is compiled against each header and must
print the same tile geometry for edge, interior and oversize tiles, ranges
1-3 and 1-16 iterations, in 1D, 2D and 3D arrays."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF_SRC = ROOT / "oracle" / "_ref" / "src"


def run(include_dir, tmp_path, name):
    exe = tmp_path / name
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(include_dir), str(ROOT / "tests" / "cpp" / "tiling_cases.cpp"),
                    "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_tile_geometry_matches_reference(tmp_path):
    if not (REF_SRC / "PSkelStencilTiling.h").is_file():
        import oracle
        oracle.build_ref()
    if not (REF_SRC / "PSkelStencilTiling.h").is_file():
        pytest.skip("the oracle's copy of the reference headers is not prepared")
    ours = run(ROOT / "include", tmp_path, "ours")
    ref = run(REF_SRC, tmp_path, "ref")
    assert ours.count("\n") > 1000
    assert ours == ref
