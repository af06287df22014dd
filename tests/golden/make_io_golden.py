"""Generate tests/golden/ref_genbc.npz: geniBC and genBC1 of the reference, run here.

fexec.py translates the reference's ``common/genibc.f`` and ``common/genbc1.f``
into numpy code; this script sets the COMMON values a single-rank compressible
run holds (nshg, ndof = 5, nsd = 3, no scalars) and the ``readarrays`` module's
nBC/iBCtmp, then stores seeded inputs and the reference's outputs:

* ``nBC`` (nshg), ``iBCtmp`` (numpbc), ``BCinp`` (numpbc, 12) -- the geombc arrays;
* ``iBC`` from geniBC and ``BC`` (nshg, 6) from genBC1 applied to genBC's gather
  ``BCtmp(:,i) = BCinp(nBC(:),i)`` (genbc.f:52-57).

The codes cover every velocity-constraint case of genBC1 (1..7) with and
without the density, temperature and pressure bits, and the two-vector cases
with the vector order flipped (a zero pivot entry, genbc1.f:70-76).

    python tests/golden/make_io_golden.py [reference phSolver directory]
"""
from __future__ import annotations

import sys
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE)]

import fexec  # noqa: E402

# the reference tree: $PHASTA_REFERENCE, else a directory "reference" beside the repository
DEFAULT_REF = Path(os.environ.get("PHASTA_REFERENCE", str(Path(__file__).resolve().parents[3] / "reference"))) / "phSolver"


def inputs(seed=20261204):
    rng = np.random.default_rng(seed)
    codes = []
    for v in range(8):
        for thermo in (0, 1, 2, 4, 6):
            codes.append((v << 3) | thermo)
    codes += [1 << 10, (1 << 10) | (7 << 3) | 2]          # periodic bits ride along
    codes = np.array(codes * 3, dtype=np.int64)           # three nodes per code
    numpbc = len(codes)
    BCinp = rng.uniform(0.2, 1.0, size=(numpbc, 12)) * rng.choice([-1.0, 1.0], size=(numpbc, 12))
    BCinp[:, 11] = 0.0                                    # no periodic rotation
    # flipped vector order for the two-constraint cases: zero the pivot entry of vector 1
    vcase = (codes >> 3) & 7
    for case, col in ((3, 3), (5, 3), (6, 4)):
        idx = np.where(vcase == case)[0][::3]
        BCinp[idx, col] = 0.0
    nshg = numpbc + 17
    nBC = np.zeros(nshg, dtype=np.int64)
    nodes = rng.permutation(nshg)[:numpbc]
    nBC[nodes] = np.arange(1, numpbc + 1)
    return nBC, codes, BCinp


def run(root: Path):
    nBC, iBCtmp, BCinp = inputs()
    nshg, numpbc = len(nBC), len(iBCtmp)
    P = fexec.Program([root / "common", root / "compressible"])
    for f in ("common/genibc.f", "common/genbc1.f"):
        P.load(root / f)
    P.module("readarrays", {"nbc": nBC.copy(), "ibctmp": iBCtmp.copy()})
    P.module("pointer_data", {})
    P.function("genibc")
    G = P.G
    G.nshg, G.numnp, G.numpbc = nshg, nshg, numpbc
    G.ndof, G.nsd, G.nsclr, G.ndofbc, G.nflow = 5, 3, 0, 6, 5
    G.necho, G.ideformwall = 3, 0
    iBC = np.zeros(nshg, dtype=np.int64)
    P.call("genibc", iBC)
    BCtmp = np.zeros((nshg, 12), order="F")
    m = nBC != 0
    BCtmp[m, :] = BCinp[nBC[m] - 1, :]
    BC = np.zeros((nshg, 6), order="F")
    P.call("genbc1", BCtmp, iBC, BC)
    return dict(nBC=nBC.astype(np.int32), iBCtmp=iBCtmp.astype(np.int32), BCinp=BCinp,
                iBC=iBC.astype(np.int32), BC=np.asarray(BC))


def main():
    root = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF
    out = run(root)
    np.savez_compressed(HERE / "ref_genbc.npz", **out)
    print("wrote", HERE / "ref_genbc.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
