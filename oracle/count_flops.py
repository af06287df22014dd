"""Exact floating-point operation counts of the reference formulation of e3 -- test
infrastructure (the oracle's element routine instantiated with a counting scalar).

The oracle restates e3.f and the routines it calls (e3ivar, getthm, getdiff, e3metric,
e3mtrx, e3conv, e3visc, e3LS/e3tau, e3massr, e3bdg, e3wmlt) statement by statement, so its
count on one element is the reference's algorithmic count for that element: every +, -, *,
/ and sqrt of two operands counts one operation.  Counted per element topology for
  res      ires = 1, iprec = 0   the residual (ItrRes of the outer residual),
  modres   ires = 2, iprec = 0   the modified residual (one ItrRes of the finite-difference
                                 Jacobian-vector product Au1MFG, au1mfg.f:72-77),
  full     ires = 3, iprec = 1   ElmMFG: both residuals and the block diagonal (e3bdg),
  bdiag    full minus ires = 3, iprec = 0: the block diagonal's share.
``python -m oracle.count_flops`` writes profiles/flops_per_element.json, which bench.py reads
for the algorithmic FP32 fraction of the element sweeps (the GPU's regrouped formulation does
less work than the reference's: the fraction is the reference's work per second).
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import pyoracle  # noqa: E402

MODES = {"res": (1, 0), "modres": (2, 0), "full": (3, 1), "full_nobd": (3, 0)}


def _sig(L):
    f = L.or_e3_flops
    dp = C.POINTER(C.c_double)
    f.argtypes = [C.POINTER(pyoracle.Common), C.c_int, C.c_int, C.c_int] + [dp] * 7
    f.restype = C.c_longlong
    g = L.or_e3_topo
    g.argtypes = [C.POINTER(pyoracle.Common), C.c_int, C.c_int, C.c_int] + [dp] * 7
    g.restype = None
    return f, g


def element_arrays(case, y, ac, lcsyst: int, e: int = 0):
    """yl, ycl, acl (nshl, 5) in element order (p, u, v, w, T) and xl (nshl, 3) of element e of a block."""
    conn = {1: case.ien, 2: case.ienh, 3: case.ienw}[lcsyst]
    nodes = np.asarray(conn[e])
    yy = np.asarray(y).reshape(5, case.nshg)
    aa = np.asarray(ac).reshape(5, case.nshg)
    order = [3, 0, 1, 2, 4]
    yl = np.ascontiguousarray(yy[order][:, nodes].T)
    al = np.ascontiguousarray(aa[order][:, nodes].T)
    xl = np.ascontiguousarray(case.x[nodes])
    return yl, yl.copy(), al, xl


def count(params: dict, lcsyst: int, ires: int, iprec: int, yl, ycl, acl, xl):
    """(flops, rl, rml, bd) of the counting instance, and the same outputs of the oracle's double instance."""
    L = pyoracle.lib()
    f, g = _sig(L)
    c = pyoracle.common(params)
    n = yl.shape[0]
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    out = [np.zeros((n, 5)), np.zeros((n, 5)), np.zeros((n, 5, 5))]
    ref = [np.zeros((n, 5)), np.zeros((n, 5)), np.zeros((n, 5, 5))]
    nf = f(C.byref(c), lcsyst, ires, iprec, d(yl), d(ycl), d(acl), d(xl), *(d(a) for a in out))
    g(C.byref(c), lcsyst, ires, iprec, d(yl), d(ycl), d(acl), d(xl), *(d(a) for a in ref))
    return int(nf), out, ref


def counts(params, case, y, ac, lcsyst):
    yl, ycl, acl, xl = element_arrays(case, y, ac, lcsyst)
    r = {k: count(params, lcsyst, ires, iprec, yl, ycl, acl, xl)[0] for k, (ires, iprec) in MODES.items()}
    r["bdiag"] = r["full"] - r["full_nobd"]
    return r


def main(out=None):
    sys.path.insert(0, str(ROOT / "tests"))
    from helpers import channel, layered
    case, p, y, ac = channel(4, ac_scale=0.05)
    res = {"tet": counts(p, case, y, ac, 1)}
    case, p, y, ac = layered(3, (1, 1, 1))
    res["hex"] = counts(p, case, y, ac, 2)
    res["wedge"] = counts(p, case, y, ac, 3)
    doc = {"what": "floating-point operations per element of the reference formulation of e3 (the oracle's "
                   "element routine with a counting scalar; + - * / sqrt each count one)",
           "command": "python -m oracle.count_flops", "per_element": res,
           "sweeps": {"ress": "tet.res", "lin": "tet.modres", "full": "tet.bdiag"}}
    path = Path(out) if out else ROOT / "profiles" / "flops_per_element.json"
    path.write_text(json.dumps(doc, indent=1) + "\n")
    return doc


if __name__ == "__main__":
    print(json.dumps(main()["per_element"], indent=1))
