"""Build the oracle (test infrastructure only) and, where the reference
sources are present, the reference's own quadrature/shape-function C code.

* ``oracle/libphoracle.so``: the C++ FP64 restatement (phasta_oracle.cpp),
  compiled with -ffp-contract=off so no multiply-add is fused;
* ``oracle/_ref/libphref_shape.so``: symtet.c, symtri.c and the
  shapeFunction sources of the reference compiled in place (with a two-line
  FCMangle.h written into oracle/_ref/include), used to pin the oracle's
  quadrature and shape tables.  Only built when the reference tree exists.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "libphoracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libphref_shape.so"
# the reference tree: $PHASTA_REFERENCE, else a directory "reference" beside the repository
REFERENCE = Path(os.environ.get("PHASTA_REFERENCE", str(HERE.parent.parent / "reference")))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def build_oracle(force: bool = False) -> Path:
    src = HERE / "phasta_oracle.cpp"
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(src.stat().st_mtime,
                                                                   (HERE / "phasta_oracle.h").stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    _run(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp), str(src),
          "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def build_reference_shape(force: bool = False) -> Path | None:
    """Compile the reference's quadrature and shape-function C sources in place."""
    common = REFERENCE / "phSolver" / "common"
    shapesrc = REFERENCE / "shapeFunction" / "src"
    if not (common / "symtet.c").exists() or not shapesrc.exists():
        return None
    if REF_LIB.exists() and not force and REF_LIB.stat().st_mtime >= Path(__file__).stat().st_mtime:
        return REF_LIB
    inc = REF_DIR / "include"
    inc.mkdir(parents=True, exist_ok=True)
    # what CMake's FortranCInterface would generate: lower-case names with a trailing underscore
    (inc / "FCMangle.h").write_text(
        "#define FortranCInterface_GLOBAL(name,NAME) name##_\n"
        "#define FortranCInterface_GLOBAL_(name,NAME) name##_\n")
    # tet/triangle rules and shapes; hex, wedge and quadrilateral rules (symhex.c, symwdg.c,
    # symquad.c, symquadw.c) with the hex/wedge shapes (shphex.c, shp6w.c -> newshape.cc)
    srcs = [common / n for n in ("symtet.c", "symtri.c", "symhex.c", "symwdg.c", "symquad.c", "symquadw.c",
                                 "shphex.c", "shp6w.c")]
    srcs += sorted(p for p in shapesrc.glob("*.c"))
    objs = []
    for s in srcs:
        o = REF_DIR / (s.stem + ".o")
        _run(["gcc", "-O2", "-fPIC", "-I", str(inc), "-I", str(shapesrc), "-c", str(s), "-o", str(o)])
        objs.append(o)
    o = REF_DIR / "newshape.o"
    _run(["g++", "-O2", "-fPIC", "-I", str(common), "-c", str(common / "newshape.cc"), "-o", str(o)])
    objs.append(o)
    _run(["g++", "-shared", "-o", str(REF_LIB), *map(str, objs), "-lm"])
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference_shape(force="--force" in sys.argv))
