"""Build the CUDA library of the hot path in place (sm_103a only).

``build()`` compiles ``csrc/*.cu`` (and the host-only ``csrc/phio.cpp``, ``csrc/reorder.cpp``) into ``phasta_gb300/libphgpu.so`` with one
``-gencode`` (compute_103a/sm_103a); the translation units are compiled in
parallel and linked with the CUDA runtime.  Nothing is installed outside the
package directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "libphgpu.so"
BUILD = PKG / "_build"
SOURCES = ["elements.cu", "nodal.cu", "solver.cu", "chunks.cu", "noalloc.cu", "sparse.cu", "tangent.cu", "topo_ress.cu",
           "learn.cu", "boundary.cu", "phio.cpp", "reorder.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build phasta_gb300")


def _flags() -> list[str]:
    # PHGPU_NVCC_FLAGS: extra flags, e.g. -DPHGPU_TOPO_LEAN_MINB=5 to compile another occupancy variant
    extra = os.environ.get("PHGPU_NVCC_FLAGS", "").split()
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                   "--expt-relaxed-constexpr", *extra]


def _compile(src: str) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), *_flags(), "-c", str(CSRC / src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.cpp")) + \
        [PKG.parent / "include" / "phgpu.h", PKG.parent / "include" / "phgpu_io.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
