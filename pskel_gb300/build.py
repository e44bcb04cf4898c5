"""Build recipe for ``libpskel_gb300.so`` (sm_103a), compiled in-tree.

Each CUDA translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
``pskel_gb300/libpskel_gb300.so``. No cmake, no torch extension machinery: the
library is a plain C-ABI shared object.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libpskel_gb300.so"

SOURCES = ["capi.cu", "life.cu", "stencil2d.cu", "stencil2d_fast.cu", "stream2d.cu", "stencil3d.cu", "stream3d_tb.cu", "noalloc.cu", "batch.cu", "mlp.cu", "tuner.cu", "selftest.cu", "outofcore.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-Xptxas",
              "-warn-spills", "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _needs(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OBJ.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        if _needs(o, [s] + headers) or extra:
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *(extra or []), "-c", str(s), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    objs = [str(OBJ / (Path(s).stem + ".o")) for s in SOURCES]
    if jobs or not LIB.exists():
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart"], check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
