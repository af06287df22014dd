"""PHASTA input/output files for the GPU path (host side of ``include/phgpu_io.h``).

The reference reads each rank's mesh from ``geombc.dat.<rank+1>`` and its state
from ``restart.<step>.<rank+1>`` (phastaIO POSIX format, readnblk.f) and writes
``restart.<step>.<rank+1>`` after a run (restar.f, Write_Restart).  This module
gives those files to the GPU path:

* ``PhastaFile`` -- openfile/readheader/readdatablock/writeheader/writedatablock;
* ``read_case`` -- geombc -> ``mesh.Case`` (geniBC, genBC1, 0-based connectivity),
  ``write_case`` -- the inverse, for synthetic cases;
* ``read_restart`` / ``write_restart`` -- y and ac in the solver's (u, v, w, p, T) order;
* ``checkphasta`` -- the largest solution difference of two case directories over
  their common time steps (checkphasta/checkphasta.cpp), with its pass/fail rule.

Every call goes through the C++ library (``csrc/phio.cpp``); nothing here
parses the files itself.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _lib as L
from .mesh import BndBlock, Case

LCSYST = {1: "tetrahedron", 2: "hexahedron", 3: "wedge"}


class PhastaIOError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"phgpu_io status {L.STATUS.get(code, code)}: {msg}")
        self.code = code


def _check(rc: int):
    if rc != L.PHGPU_OK:
        raise PhastaIOError(rc, L.lib().phgpu_io_last_error().decode())


def _b(s: str | os.PathLike) -> bytes:
    return os.fsencode(str(s))


class PhastaFile:
    """One open PHASTA file (the phastaIO POSIX calls)."""

    def __init__(self, path, mode: str = "read", iotype: str = "binary"):
        self.lib = L.lib()
        self.mode, self.iotype = mode, iotype
        fd = C.c_int(0)
        _check(self.lib.phgpu_io_openfile(_b(path), mode.encode(), C.byref(fd)))
        self.fd = fd.value

    def close(self):
        if self.fd:
            fd, self.fd = self.fd, 0
            _check(self.lib.phgpu_io_closefile(fd, self.mode.encode()))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def readheader(self, key: str, nitems: int, datatype: str = "integer"):
        """Header integers of ``key``, or None when the key is not in the file."""
        v = np.zeros(max(nitems, 1), dtype=np.int32)
        rc = self.lib.phgpu_io_readheader(self.fd, key.encode(), L.iptr(v), nitems, datatype.encode(),
                                          self.iotype.encode())
        if rc == L.PHGPU_ERR_NOTFOUND:
            return None
        _check(rc)
        return v[:nitems]

    def readdatablock(self, key: str, nitems: int, datatype: str = "double"):
        a = np.zeros(nitems, dtype=np.int32 if datatype.startswith("int") else np.float64)
        _check(self.lib.phgpu_io_readdatablock(self.fd, key.encode(), a.ctypes.data_as(C.c_void_p), nitems,
                                               datatype.encode(), self.iotype.encode()))
        return a

    def writeheader(self, key: str, values, ndata: int, datatype: str = "double"):
        v = np.ascontiguousarray(np.asarray(values, dtype=np.int32).reshape(-1))
        _check(self.lib.phgpu_io_writeheader(self.fd, key.encode(), L.iptr(v) if v.size else None, v.size,
                                             ndata, datatype.encode(), self.iotype.encode()))

    def writedatablock(self, key: str, values, datatype: str = "double"):
        a = np.ascontiguousarray(np.asarray(values, dtype=np.int32 if datatype.startswith("int") else np.float64)
                                 .reshape(-1))
        _check(self.lib.phgpu_io_writedatablock(self.fd, key.encode(), a.ctypes.data_as(C.c_void_p), a.size,
                                                datatype.encode(), self.iotype.encode()))

    def write(self, key: str, header, values, datatype: str):
        values = np.asarray(values)
        self.writeheader(key, header, values.size, datatype)
        self.writedatablock(key, values, datatype)

    def writestring(self, text: str):
        _check(self.lib.phgpu_io_writestring(self.fd, text.encode()))


# ---- restart files ---------------------------------------------------------------------------

def write_restart(dirname, step: int, y: np.ndarray, ac: np.ndarray, rank: int = 0) -> Path:
    """restart.<step>.<rank+1>; y, ac of shape (ndof, nshg) in the solver's order."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    ac = np.ascontiguousarray(ac, dtype=np.float64)
    ndof, nshg = y.shape
    _check(L.lib().phgpu_io_write_restart(_b(dirname), rank, step, nshg, ndof, L.dptr(y), L.dptr(ac)))
    return Path(dirname) / f"restart.{step}.{rank + 1}"


def read_restart(dirname, step: int, nshg: int, ndof: int = 5, rank: int = 0):
    """(y, ac, lstep) from restart.<step>.<rank+1>, arrays (ndof, nshg) in the solver's order."""
    y = np.zeros((ndof, nshg))
    ac = np.zeros((ndof, nshg))
    lstep = C.c_int(0)
    _check(L.lib().phgpu_io_read_restart(_b(dirname), rank, step, nshg, ndof, L.dptr(y), L.dptr(ac),
                                         C.byref(lstep)))
    return y, ac, lstep.value


def checkphasta(left, right, tolerance: float, nparts: int = 1):
    """(max difference, common time steps, passed) as checkphasta reports and exits."""
    m = np.zeros(1)
    n = C.c_int(0)
    _check(L.lib().phgpu_io_checkphasta(_b(left), _b(right), nparts, L.dptr(m), C.byref(n)))
    return float(m[0]), n.value, not (m[0] > tolerance)


# ---- geombc ----------------------------------------------------------------------------------

def read_geombc(dirname, rank: int = 0, ndof: int = 5) -> dict:
    """The arrays of geombc.dat.<rank+1> as the reference holds them after readnblk
    (1-based connectivity, Fortran layouts reshaped to numpy (rows, columns))."""
    lib = L.lib()
    h = C.c_void_p()
    _check(lib.phgpu_io_geombc_open(_b(dirname), rank, ndof, C.byref(h)))
    try:
        info = L.GeombcInfo()
        _check(lib.phgpu_io_geombc_info(h, C.byref(info)))
        I = {k: getattr(info, k) for k, _ in L.GeombcInfo._fields_}
        x = np.zeros(I["numnp"] * I["nsd"])
        nBC = np.zeros(I["nshg"], np.int32)
        iper = np.zeros(I["nshg"], np.int32)
        iBCtmp = np.zeros(max(I["numpbc"], 1), np.int32)
        BCinp = np.zeros(max(I["numpbc"] * I["nbccols"], 1))
        _check(lib.phgpu_io_geombc_arrays(h, L.dptr(x), L.iptr(nBC), L.iptr(iBCtmp), L.dptr(BCinp), L.iptr(iper)))
        out = dict(info=I, x=x.reshape(I["nsd"], I["numnp"]).T, nBC=nBC, iper=iper,
                   iBCtmp=iBCtmp[:I["numpbc"]],
                   BCinp=BCinp[:I["numpbc"] * I["nbccols"]].reshape(I["nbccols"], I["numpbc"]).T,
                   interior=[], boundary=[])
        for b in range(I["nelblk"]):
            blk = L.TopBlock()
            _check(lib.phgpu_io_geombc_interior(h, b, C.byref(blk), None))
            ien = np.zeros(max(blk.neltp * blk.nshl, 1), np.int32)
            _check(lib.phgpu_io_geombc_interior(h, b, C.byref(blk), L.iptr(ien)))
            t = {k: getattr(blk, k) for k, _ in L.TopBlock._fields_}
            out["interior"].append((t, ien[:blk.neltp * blk.nshl].reshape(blk.nshl, blk.neltp).T))
        for b in range(I["nelblb"]):
            blk = L.TopBlock()
            _check(lib.phgpu_io_geombc_boundary(h, b, C.byref(blk), None, None, None))
            ne = blk.neltp
            ienb = np.zeros(max(ne * blk.nshl, 1), np.int32)
            ibcb = np.zeros(max(ne * 2, 1), np.int32)
            bcb = np.zeros(max(ne * blk.nshlb * (ndof + 1), 1))
            _check(lib.phgpu_io_geombc_boundary(h, b, C.byref(blk), L.iptr(ienb), L.iptr(ibcb), L.dptr(bcb)))
            t = {k: getattr(blk, k) for k, _ in L.TopBlock._fields_}
            out["boundary"].append((t, ienb[:ne * blk.nshl].reshape(blk.nshl, ne).T,
                                    ibcb[:ne * 2].reshape(2, ne).T,
                                    bcb[:ne * blk.nshlb * (ndof + 1)].reshape(ndof + 1, blk.nshlb, ne).transpose(2, 1, 0)))
        return out
    finally:
        lib.phgpu_io_geombc_free(h)


def boundary_conditions(nBC, iBCtmp, BCinp, ndof: int = 5):
    """(iBC, BC (ndof+1, nshg)) by geniBC and genBC1."""
    lib = L.lib()
    nBC = np.ascontiguousarray(nBC, dtype=np.int32)
    iBCtmp = np.ascontiguousarray(iBCtmp, dtype=np.int32)
    nshg, numpbc = nBC.size, iBCtmp.size
    iBC = np.zeros(nshg, np.int32)
    _check(lib.phgpu_io_genibc(nshg, numpbc, L.iptr(nBC), L.iptr(iBCtmp) if numpbc else None, L.iptr(iBC)))
    B = np.ascontiguousarray(np.asarray(BCinp, dtype=np.float64).T).reshape(-1)
    ld = np.asarray(BCinp).shape[1] if numpbc else ndof + 7
    BC = np.zeros((ndof + 1) * nshg)
    _check(lib.phgpu_io_genbc(nshg, numpbc, ndof, L.iptr(nBC), L.dptr(B) if numpbc else None, ld,
                              L.iptr(iBC), L.dptr(BC)))
    return iBC, BC.reshape(ndof + 1, nshg)


def _min_edge(x, blocks):
    h = np.inf
    for ien in blocks:
        if not len(ien):
            continue
        p = x[ien]
        for a in range(ien.shape[1]):
            for b in range(a + 1, ien.shape[1]):
                h = min(h, float(np.min(np.linalg.norm(p[:, a] - p[:, b], axis=1))))
    return h


def read_case(dirname, rank: int = 0) -> Case:
    """geombc.dat.<rank+1> as a ``mesh.Case``: linear tets, hexes and wedges; boundary tets with
    their face first, and boundary hexes and wedges as ``mesh.BndBlock``s (a wedge block's
    boundary rule follows its face's node count, 3 or 4, as elmmfg.f:187 does; 0-based
    connectivity)."""
    g = read_geombc(dirname, rank)
    ien = {1: [], 2: [], 3: []}
    for t, e in g["interior"]:
        if t["lcsyst"] not in ien or t["ipordl"] != 1 or t["nshl"] != t["nenl"]:
            raise PhastaIOError(L.PHGPU_ERR_UNSUPPORTED,
                                f"interior block lcsyst {t['lcsyst']}, order {t['ipordl']}, nshl {t['nshl']}")
        ien[t["lcsyst"]].append(np.abs(e) - 1)
    ienb, ibcb, bcb, bnd = [], [], [], {}
    for t, e, codes, vals in g["boundary"]:
        shape = (t["lcsyst"], t["nshl"], t["nshlb"])
        if t["ipordl"] != 1 or shape not in ((1, 4, 3), (2, 8, 4), (3, 6, 3), (3, 6, 4)):
            raise PhastaIOError(L.PHGPU_ERR_UNSUPPORTED, f"boundary block lcsyst {t['lcsyst']}, nshl {t['nshl']}, "
                                                         f"nshlb {t['nshlb']}, order {t['ipordl']}")
        if t["lcsyst"] == 1:
            ienb.append(np.abs(e) - 1)
            ibcb.append(codes)
            bcb.append(vals)
        else:
            lc = 2 if t["lcsyst"] == 2 else (3 if t["nshlb"] == 3 else 4)
            bnd.setdefault(lc, []).append((np.abs(e) - 1, codes, vals))
    iBC, BC = boundary_conditions(g["nBC"], g["iBCtmp"], g["BCinp"])
    x = np.ascontiguousarray(g["x"])
    cat = lambda parts, n: (np.concatenate(parts) if parts else np.zeros((0, n))).astype(np.int32)  # noqa: E731
    tets, hexes, wedges = cat(ien[1], 4), cat(ien[2], 8), cat(ien[3], 6)
    bblocks = [BndBlock(lc, np.concatenate([b[0] for b in v]).astype(np.int32),
                        np.concatenate([b[1] for b in v]).astype(np.int32), np.concatenate([b[2] for b in v]))
               for lc, v in sorted(bnd.items())]
    return Case(nshg=g["info"]["nshg"], x=x, ien=tets, ienb=cat(ienb, 4), iBCB=cat(ibcb, 2),
                BCB=(np.concatenate(bcb) if bcb else np.zeros((0, 3, 6))), iBC=iBC, BC=BC,
                iper=(g["iper"] - 1).astype(np.int32), h=_min_edge(x, [tets, hexes, wedges]),
                meta={"source": str(dirname)}, ienh=hexes, ienw=wedges, bnd=bblocks)


def _bcinp(case: Case):
    """BCinp rows (D T P c11 c12 c13 M1 c21 c22 c23 M2 theta) that genBC1 turns back into
    the case's BC: velocity codes 0 and 7 (c1 = velocity, M1 = 1) and the single-component
    codes 1, 2, 4 (pivot 1)."""
    iBC, BC = case.iBC, case.BC
    nodes = np.where(iBC != 0)[0]
    rows = np.zeros((len(nodes), 12))
    code = iBC[nodes]
    bc = BC[:, nodes]
    rows[:, 0] = np.where(code & 1, bc[0], 0.0)
    rows[:, 1] = np.where(code & 2, bc[1], 0.0)
    rows[:, 2] = np.where(code & 4, bc[0], 0.0)
    v = (code >> 3) & 7
    if np.any(np.isin(v, (3, 5, 6))):
        raise PhastaIOError(L.PHGPU_ERR_UNSUPPORTED, "two-component velocity constraints cannot be written")
    w = v == 7
    rows[w, 3:6] = bc[2:5, w].T
    rows[w, 6] = 1.0
    for case_v, piv, o1, o2 in ((1, 3, 4, 5), (2, 4, 3, 5), (4, 5, 3, 4)):
        w = v == case_v
        rows[w, piv] = 1.0
        rows[w, o1] = bc[3, w]
        rows[w, o2] = bc[4, w]
        rows[w, 6] = bc[2, w] / (1.0 + bc[3, w] ** 2 + bc[4, w] ** 2)
    nBC = np.zeros(case.nshg, np.int32)
    nBC[nodes] = np.arange(1, len(nodes) + 1)
    return nBC, code.astype(np.int32), rows


def write_case(case: Case, dirname, rank: int = 0) -> Path:
    """geombc.dat.<rank+1> holding the headers readnblk reads (one block per topology)."""
    path = Path(dirname) / f"geombc.dat.{rank + 1}"
    nBC, codes, rows = _bcinp(case)
    blocks = [(case.ien, 1), (case.ienh, 2), (case.ienw, 3)]
    blocks = [(np.asarray(e, np.int32) + 1, lc) for e, lc in blocks if len(e)]
    nen = max(e.shape[1] for e, _ in blocks)
    with PhastaFile(path, "write") as f:
        f.writestring("# PHASTA Input File Version 2.0\n")
        f.write("byteorder magic number", [362436], [362436], "integer")
        counts = [("number of nodes", case.nshg), ("number of modes", case.nshg),
                  ("number of interior elements", sum(len(e) for e, _ in blocks)),
                  ("number of boundary elements", case.nbelem + sum(len(b.ien) for b in case.bnd)),
                  ("maximum number of element nodes", nen),
                  ("number of interior tpblocks", len(blocks)),
                  ("number of boundary tpblocks", (1 if case.nbelem else 0) + len(case.bnd)),
                  ("number of nodes with Dirichlet BCs", len(codes)), ("number of shape functions", nen)]
        for k, v in counts:
            f.writeheader(k, [v], 0, "integer")
        f.write("co-ordinates", [case.nshg, 3], np.asarray(case.x).T, "double")
        for e, lc in blocks:
            ne, nshl = e.shape
            f.write(f"connectivity interior linear {LCSYST[lc]}", [ne, nshl, 1, nshl, 0, 0, lc], e.T, "integer")
        f.write("bc mapping array", [case.nshg], nBC, "integer")
        f.write("bc codes array", [len(codes)], codes, "integer")
        f.write("boundary condition array", [rows.size], rows.T, "double")
        f.write("periodic masters array", [case.nshg], np.asarray(case.iper, np.int32) + 1, "integer")
        if case.nbelem:
            ne = case.nbelem
            h = [ne, 4, 1, 4, 3, 3, 1, 6]
            f.write("connectivity boundary linear tetrahedron", h, (np.asarray(case.ienb, np.int32) + 1).T, "integer")
            f.write("nbc codes linear tetrahedron", h, np.asarray(case.iBCB, np.int32).T, "integer")
            f.write("nbc values linear tetrahedron", h, np.asarray(case.BCB)[:, 0, :].T, "double")
        # boundary hexes and wedges: header (neltp, nenl, ipordl, nshl, nshlb, nenbl, lcsyst, numnbc), the
        # lcsyst of the element topology (a wedge block's face size tells its boundary rule)
        for b in case.bnd:
            ne, nshl, nb = len(b.ien), b.nshl, b.nshlb
            lc = 2 if b.lcsyst == 2 else 3
            h = [ne, nshl, 1, nshl, nb, nb, lc, 6]
            name = LCSYST[lc]
            f.write(f"connectivity boundary linear {name}", h, (np.asarray(b.ien, np.int32) + 1).T, "integer")
            f.write(f"nbc codes linear {name}", h, np.asarray(b.iBCB, np.int32).T, "integer")
            f.write(f"nbc values linear {name}", h, np.asarray(b.BCB)[:, 0, :].T, "double")
    return path
