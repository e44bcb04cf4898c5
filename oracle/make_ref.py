"""Build recipe for ``oracle/_ref``: the reference's own ``runIterativeCPU``
(and its ``runIterativeGPU``, to measure the library beside it).

Test infrastructure only. The product never imports, links or runs anything
under ``oracle/``; tests, ``__graft_entry__.smoke()`` and the CPU-baseline and
reference legs of ``bench.py`` use it as the checker and the baseline.

The reference (PSkel, header-only C++) does not compile for the CPU as shipped:
``PSkelArray.hpp`` defines three groups of CUDA-only members outside any
``#ifdef PSKEL_CUDA`` guard (lines 209-230 ``hostAllocPinned``, 278-284
``cudaHostMemCopy``, 501-509 ``copyToDevicePinned``/``copyFromDevicePinned``),
uses ``memcpy`` without ``<cstring>`` (line 412), unconditionally includes
``<tbb/scalable_allocator.h>`` (``PSkel.h:80``) and ``<xmmintrin.h>``
(``PSkelArray.hpp:42``, only for ``_mm_malloc``/``_mm_free``).

This script therefore:
  1. copies the reference headers into ``oracle/_ref/src`` (git-ignored output
     directory; nothing of the reference is committed),
  2. wraps exactly those three line ranges of the copy in ``#ifdef PSKEL_CUDA``
     after checking the sha256 of the original file, so a different reference
     revision is refused instead of being patched blindly, and qualifies the
     two device accesses of lines 345 and 642 (``width``/``depth`` of a
     dependent base) with ``this->`` so the copy also compiles under nvcc with
     ``PSKEL_CUDA`` (to show that user code compiles against it, and for the
     GPU runner below),
  3. writes two shim headers (``tbb/scalable_allocator.h`` over malloc/free and
     ``xmmintrin.h`` over posix_memalign, which also makes the build portable
     to aarch64 hosts),
  4. compiles ``oracle/ref_runner.cpp`` against the copy with
     ``g++ -O3 -ffp-contract=off -fopenmp -DPSKEL_OMP`` into
     ``oracle/_ref/pskel_ref``, and ``oracle/ref_runner_gpu.cu`` (the
     reference's own ``runIterativeGPU``, measured beside the library) with
     ``nvcc -O3 -DPSKEL_CUDA`` for sm_103a into ``oracle/_ref/pskel_ref_gpu``
     when nvcc is present.

Step 1-3 need the reference tree (the ``PSKEL_REFERENCE`` environment
variable, else a ``reference`` directory beside this repository's root). Step 4 only needs ``oracle/_ref/src``,
so on a machine without the reference the previously prepared copy is compiled.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC = OUT / "src"
SHIM = OUT / "shim"
BIN = OUT / "pskel_ref"
GPU_BIN = OUT / "pskel_ref_gpu"

# sha256 of the reference PSkelArray.hpp the line ranges below were read from.
ARRAY_HPP_SHA256 = "eee8c8e0c3e492be63452c199138c7b73d5ac7af7b0a2e8527e2e8d8c6d06fe6"
# 1-based inclusive line ranges of PSkelArray.hpp that only make sense with CUDA.
CUDA_ONLY_RANGES = [(209, 230), (278, 284), (501, 509)]
# 1-based lines of PSkelArray.hpp whose device access needs this-> qualified members.
UNQUALIFIED_LINES = [345, 642]

SHIM_TBB = """// Shim for the oracle build: PSkel.h includes this header unconditionally.
#pragma once
#include <cstdlib>
inline void* scalable_malloc(size_t n) { return std::malloc(n); }
inline void scalable_free(void* p) { std::free(p); }
"""

SHIM_XMM = """// Shim for the oracle build: PSkelArray.hpp needs only _mm_malloc/_mm_free.
#pragma once
#include <cstdlib>
inline void* _mm_malloc(size_t n, size_t a) {
  void* p = nullptr;
  if (a < sizeof(void*)) a = sizeof(void*);
  if (posix_memalign(&p, a, n ? n : a)) return nullptr;
  return p;
}
inline void _mm_free(void* p) { std::free(p); }
"""


def reference_include() -> Path | None:
    """The reference's include/ directory: $PSKEL_REFERENCE, else a checkout
    named ``reference`` next to this repository (the build layout here)."""
    env = os.environ.get("PSKEL_REFERENCE")
    root = Path(env) if env else HERE.parent.parent / "reference"
    inc = root / "include"
    return inc if (inc / "PSkelStencil.hpp").is_file() else None


def prepare_overlay(inc: Path) -> None:
    """Copy the reference headers and guard the CUDA-only line ranges."""
    SRC.mkdir(parents=True, exist_ok=True)
    for f in sorted(inc.iterdir()):
        if f.suffix in (".h", ".hpp"):
            shutil.copyfile(f, SRC / f.name)
    arr = SRC / "PSkelArray.hpp"
    raw = (inc / "PSkelArray.hpp").read_bytes()
    digest = hashlib.sha256(raw).hexdigest()
    if digest != ARRAY_HPP_SHA256:
        raise RuntimeError(f"unexpected PSkelArray.hpp revision (sha256 {digest}); "
                           "line ranges of the overlay were read from another revision")
    lines = raw.decode("latin-1").split("\n")
    # Array::operator() and Array3D::operator() (lines 345 and 642) name the
    # dependent base members width/depth without this->, which nvcc rejects
    # once PSKEL_CUDA compiles the device branch: qualify them, nothing else.
    unq = "return this->deviceArray[(h*width+w)*depth+d];"
    hits = [i for i, l in enumerate(lines) if l.strip() == unq]
    if [i + 1 for i in hits] != UNQUALIFIED_LINES:
        raise RuntimeError(f"unexpected PSkelArray.hpp: unqualified device accesses at {[i + 1 for i in hits]}")
    for i in hits:
        lines[i] = lines[i].replace(unq, "return this->deviceArray[(h*this->width+w)*this->depth+d];")
    for lo, hi in sorted(CUDA_ONLY_RANGES, reverse=True):
        lines.insert(hi, "#endif /* oracle overlay */")
        lines.insert(lo - 1, "#ifdef PSKEL_CUDA /* oracle overlay */")
    arr.write_bytes("\n".join(lines).encode("latin-1"))
    (SHIM / "tbb").mkdir(parents=True, exist_ok=True)
    (SHIM / "tbb" / "scalable_allocator.h").write_text(SHIM_TBB)
    (SHIM / "xmmintrin.h").write_text(SHIM_XMM)


def compile_runner() -> Path:
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fopenmp", "-DPSKEL_OMP",
           "-include", "cstring", "-I", str(SHIM), "-I", str(SRC),
           "-w", str(HERE / "ref_runner.cpp"), "-o", str(BIN)]
    subprocess.run(cmd, check=True)
    return BIN


def gpu_runner_cmd() -> list[str]:
    """nvcc command of ``pskel_ref_gpu``: the reference's GPU path as its own
    build would compile it (``PSKEL_CUDA``, nvcc's default contraction)."""
    return ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3", "-DPSKEL_CUDA",
            "-DPSKEL_OMP", "-Xcompiler", "-fopenmp", "-include", "cstring", "-I", str(SHIM), "-I", str(SRC),
            "-w", str(HERE / "ref_runner_gpu.cu"), "-o", str(GPU_BIN), "-lgomp"]


def build(require: bool = False) -> Path | None:
    """Prepare (when the reference tree is present) and compile ``pskel_ref``
    and, when nvcc is on the path, ``pskel_ref_gpu`` (both at once)."""
    inc = reference_include()
    if inc is not None:
        prepare_overlay(inc)
    if not (SRC / "PSkelStencil.hpp").is_file():
        if require:
            raise RuntimeError("reference headers unavailable: no overlay copy in oracle/_ref/src")
        return None
    gpu = subprocess.Popen(gpu_runner_cmd()) if shutil.which("nvcc") else None
    try:
        path = compile_runner()
    finally:
        if gpu is not None and gpu.wait() != 0:
            print("oracle: pskel_ref_gpu did not compile; the reference GPU comparison is skipped", file=sys.stderr)
    return path


if __name__ == "__main__":
    path = build(require=True)
    print(path)
    sys.exit(0)
