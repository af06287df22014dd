"""Generate tests/golden/tet_tables.json from the reference's own C sources.

Runs in a container that holds the reference tree: oracle/build_oracle.py
compiles symtet.c, symtri.c and shapeFunction/src/*.c of the reference in
place into oracle/_ref/libphref_shape.so; this script calls
symtet/symtri (the quadrature rules genint.f uses) and TetShapeAndDrv (the
shape functions genshp.f/genshpb.f tabulate), applies genint.f:72-73 and
genshp.f:32-35, and writes the tables the element routines read.

    python tests/golden/make_tables.py
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.build_oracle import build_reference_shape  # noqa: E402


def main():
    so = build_reference_shape()
    if so is None:
        raise SystemExit("reference sources not found")
    L = C.CDLL(str(so))
    D = C.c_double
    out = {}
    # interior: 4-point tet rule
    n, err = C.c_int(4), C.c_int(0)
    pt, wt = (D * 16)(), (D * 4)()
    L.symtet_(C.byref(n), pt, wt, C.byref(err))
    shp, shgl, qwt = [], [], []
    for q in range(4):
        par = (D * 3)(pt[4 * q], pt[4 * q + 1], pt[4 * q + 2])
        N, dN = (D * 4)(), (D * 12)()
        L.TetShapeAndDrv(1, par, N, dN)
        shp.append([N[a] for a in range(4)])
        shgl.append([[dN[3 * a + i] / 2.0 for a in range(4)] for i in range(3)])
        qwt.append((4.0 / 3.0) * wt[q])
    out["shp"], out["shgl"], out["Qwt"] = shp, shgl, qwt
    # boundary: 3-point triangle rule on the tet face
    n = C.c_int(3)
    pt, wt = (D * 12)(), (D * 3)()
    L.symtri_(C.byref(n), pt, wt, C.byref(err))
    shpb, shglb, qwtb = [], [], []
    for q in range(3):
        par = (D * 3)(pt[4 * q], pt[4 * q + 1], pt[4 * q + 2])
        N, dN = (D * 4)(), (D * 12)()
        L.TetShapeAndDrv(1, par, N, dN)
        shpb.append([N[a] for a in range(4)])
        shglb.append([[dN[3 * a + i] / 2.0 for a in range(4)] for i in range(3)])
        qwtb.append(2.0 * wt[q])
    out["shpb"], out["shglb"], out["Qwtb"] = shpb, shglb, qwtb
    out["source"] = "reference symtet.c, symtri.c, shapeFunction/src (TetShapeAndDrv), genint.f:72-73, genshp.f:32-35"
    p = Path(__file__).resolve().parent / "tet_tables.json"
    p.write_text(json.dumps(out, indent=1))
    print(p)
    topo = {}
    # hex: 8-point rule of symhex.c (genint.f:86-99, no weight scaling), shapes of shphex.c (genshp.f)
    # wedge: 6-point rule of symwdg.c (genint.f:312-317), shapes of shp6w.c; no gradient scaling for either
    for name, rule, shape, nq, nen in (("hex", L.symhex_, L.shphex_, 8, 8), ("wedge", L.symwdg_, L.shp6w_, 6, 6)):
        n = C.c_int(nq)
        pt, wt = (D * (4 * nq))(), (D * nq)()
        rule(C.byref(n), pt, wt, C.byref(err))
        shp, shgl, qwt, pts = [], [], [], []
        for q in range(nq):
            par = (D * 3)(pt[4 * q], pt[4 * q + 1], pt[4 * q + 2])
            N, dN = (D * nen)(), (D * (3 * nen))()
            shape(C.byref(C.c_int(1)), par, N, dN)
            shp.append([N[a] for a in range(nen)])
            shgl.append([[dN[3 * a + i] for a in range(nen)] for i in range(3)])
            qwt.append(wt[q])
            pts.append([pt[4 * q + k] for k in range(4)])
        topo[name] = {"shp": shp, "shgl": shgl, "Qwt": qwt, "Qpt": pts}
    # boundary elements (genint.f:119-142, 302-345; genshpb.f; shapes unscaled): lcsyst 2, the hex
    # with its zeta = -1 quadrilateral face (symquad.c); lcsyst 3, the wedge with its triangle
    # face (symtri.c, the last point moved first, zeta = -1, weights in symtri's order);
    # lcsyst 4, the wedge with a quadrilateral face (symquadw.c)
    def bnd(rule, shape, nq, nen, reorder_tri=False):
        n = C.c_int(nq)
        pt, wt = (D * (4 * nq))(), (D * nq)()
        rule(C.byref(n), pt, wt, C.byref(err))
        pts = [[pt[4 * q + k] for k in range(4)] for q in range(nq)]
        if reorder_tri:
            pts = [pts[nq - 1]] + pts[: nq - 1]
            pts = [[p[0], p[1], -1.0, -1.0] for p in pts]
        shpb, shglb = [], []
        for q in range(nq):
            par = (D * 3)(*pts[q][:3])
            N, dN = (D * nen)(), (D * (3 * nen))()
            shape(C.byref(C.c_int(1)), par, N, dN)
            shpb.append([N[a] for a in range(nen)])
            shglb.append([[dN[3 * a + i] for a in range(nen)] for i in range(3)])
        return {"shpb": shpb, "shglb": shglb, "Qwtb": [wt[q] for q in range(nq)], "Qptb": pts}
    topo["hex_quad_b"] = bnd(L.symquad_, L.shphex_, 4, 8)
    topo["wedge_tri_b"] = bnd(L.symtri_, L.shp6w_, 3, 6, reorder_tri=True)
    topo["wedge_quad_b"] = bnd(L.symquadw_, L.shp6w_, 4, 6)
    topo["source"] = ("reference symhex.c, symwdg.c, symquad.c, symtri.c, symquadw.c, shphex.c, shp6w.c -> "
                      "newshape.cc; genint.f, genshp.f, genshpb.f")
    p2 = Path(__file__).resolve().parent / "topo_tables.json"
    p2.write_text(json.dumps(topo, indent=1))
    print(p2)


if __name__ == "__main__":
    main()
