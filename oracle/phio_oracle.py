"""Oracle (test infrastructure): PHASTA's POSIX file format and the compressible solver's
restart/geombc call sequences, restated in Python over byte buffers.

Only the tests use this module, as the checker of the C++ implementation in
``phasta_gb300/csrc/phio.cpp``.  Each function cites the reference code it
restates (paths within the PHASTA project):

* ``key_match``      -- cscompare, phastaIO/phastaIO.cc:179-195
* ``header_bytes``   -- writeHeader, phastaIO/phastaIO.cc:1624-1644
* ``block_bytes``    -- writeDataBlock, phastaIO/phastaIO.cc:1819-1850
* ``Reader``         -- readHeader / readDataBlock, phastaIO/phastaIO.cc:197-306, 1450-1481,
                        with the header bookkeeping of readheader/readdatablock :1271-1448, 1483-1622
* ``restart_bytes``  -- Write_Restart, phSolver/common/new_interface.c:240-330, after
                        restar('out '), phSolver/common/restar.f:53-80
* ``read_restart``   -- readnblk.f:480-545 and restar('in  '), restar.f:34-49
* ``geombc_bytes`` / ``read_geombc`` -- the headers readnblk.f:112-385, genblkPosix.f and
                        genbkbPosix.f read, in their order
* ``genibc``, ``genbc1`` -- phSolver/common/genibc.f:44-47, genbc.f:52-57 and genbc1.f

The reference's phastaIO library cannot be built here (it needs MPI); the format is
pinned by this restatement, and geniBC/genBC1 against the reference's Fortran executed
through the translator (tests/golden/ref_genbc.npz).
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = 362436
_SEP = " ,;<>"


def key_match(phrase: str, token: str) -> bool:
    a, b = phrase, token
    i = j = 0

    def skip(s, k):
        while k < len(s) and s[k] == " ":
            k += 1
        return k

    i, j = skip(a, i), skip(b, j)
    while i < len(a) and j < len(b) and b[j] != "?" and a[i].lower() == b[j].lower():
        i, j = skip(a, i + 1), skip(b, j + 1)
    return i >= len(a) or a[i] == "?"


def _first_word(s: str) -> str:
    return s.split(" ")[0] if s else ""


def _binary(iotype: str) -> bool:
    return key_match(_first_word(iotype), "binary")


def _tsize(datatype: str) -> int:
    t = _first_word(datatype)
    return 4 if key_match("integer", t) else 8 if key_match("double", t) else 0


def header_bytes(key: str, values, ndata: int, datatype: str, iotype: str = "binary") -> bytes:
    nl = 1 if ndata > 0 else 0
    size = _tsize(datatype) * ndata + nl if _binary(iotype) else ndata
    return (f"{key} : < {size} > " + "".join(f"{int(v)} " for v in values) + "\n").encode()


def block_bytes(values, datatype: str, iotype: str = "binary") -> bytes:
    isint = _tsize(datatype) == 4
    arr = np.asarray(values, dtype=np.int32 if isint else np.float64).reshape(-1)
    if _binary(iotype):
        return arr.tobytes() + b"\n"
    fmt = "%d\n" if isint else "%f\n"
    return "".join(fmt % v for v in arr.tolist()).encode()


class Reader:
    """A phastaIO reader over a byte buffer (one open file)."""

    def __init__(self, data: bytes, native="<"):
        self.d = data
        self.pos = 0
        self.swap = False
        self.native = native

    def _line(self):
        """fgets: up to 1023 bytes or through the next newline; None at end of data."""
        if self.pos >= len(self.d):
            return None
        end = self.d.find(b"\n", self.pos, self.pos + 1023)
        end = self.pos + 1023 if end < 0 else end + 1
        end = min(end, len(self.d))
        s = self.d[self.pos:end]
        self.pos = end
        return s.decode("latin-1")

    def header(self, phrase: str, nitems: int, iotype: str = "binary"):
        """Header integers of phrase, or None; a failed search leaves the position unchanged."""
        start, swap = self.pos, self.swap
        r = self._search(phrase, nitems, iotype)
        if r is None:
            self.pos = start
            self.swap = swap or self.swap
        return r

    def _search(self, phrase: str, nitems: int, iotype: str):
        binary = _binary(iotype)
        rewinds = 0
        line = self._line()
        if line is None:
            self.pos, rewinds = 0, 1
            line = self._line() or ""
        while rewinds < 2:
            cut = line.find("#")
            text = line if cut < 0 else line[:cut]
            if line and line[0] != "\n" and text:
                stripped = text.lstrip(":")
                k = stripped.find(":")
                key = stripped if k < 0 else stripped[:k]
                rest = "" if k < 0 else stripped[k + 1:]
                fields = [f for f in _split(rest)]
                if key_match(phrase, key):
                    return [int(_atoi(f)) for f in fields[1:1 + nitems]]
                if key_match(key, "byteorder magic number"):
                    if binary:
                        v = struct.unpack(self.native + "i", self.d[self.pos:self.pos + 4])[0]
                        self.pos += 5
                        if v != MAGIC:
                            self.swap = True
                    else:
                        line2 = self._line()
                        del line2
                else:
                    skip = _atoi(fields[0])
                    if binary:
                        self.pos += skip
                    else:
                        for _ in range(skip):
                            self._line()
            line = self._line()
            if line is None:
                self.pos, rewinds = 0, rewinds + 1
                line = self._line() or ""
        return None

    def block(self, n: int, datatype: str, iotype: str = "binary"):
        isint = _tsize(datatype) == 4
        if _binary(iotype):
            ts = 4 if isint else 8
            raw = self.d[self.pos:self.pos + ts * n]
            self.pos += ts * n + 1
            order = (">" if self.native == "<" else "<") if self.swap else self.native
            return np.frombuffer(raw, dtype=np.dtype(("i4" if isint else "f8")).newbyteorder(order)).astype(
                np.int32 if isint else np.float64)
        out = [(int if isint else float)(self._line().strip()) for _ in range(n)]
        return np.array(out, dtype=np.int32 if isint else np.float64)


def _split(s: str):
    out, cur = [], ""
    for c in s:
        if c in _SEP:
            if cur:
                out.append(cur)
            cur = ""
        else:
            cur += c
    if cur:
        out.append(cur)
    return out


def _atoi(s: str) -> int:
    s = s.lstrip(" \t\n")
    sign, k = 1, 0
    if k < len(s) and s[k] in "+-":
        sign, k = (-1 if s[k] == "-" else 1), k + 1
    v = 0
    while k < len(s) and s[k].isdigit():
        v = 10 * v + int(s[k])
        k += 1
    return sign * v


# ---- restart -------------------------------------------------------------------------------

def _file_order(y):
    """(ndof, nshg) solver order (u, v, w, p, T) -> file order (p, u, v, w, T)."""
    y = np.asarray(y, dtype=np.float64)
    return np.concatenate([y[3:4], y[0:3], y[4:]], axis=0)


def _solver_order(q):
    return np.concatenate([q[1:4], q[0:1], q[4:]], axis=0)


def restart_bytes(y, ac, stepno: int) -> bytes:
    y = np.asarray(y, dtype=np.float64)
    ndof, nshg = y.shape
    out = header_bytes("byteorder magic number", [MAGIC], 1, "integer") + block_bytes([MAGIC], "integer")
    for key, v in (("solution", y), ("time derivative of solution", ac)):
        out += header_bytes(key, [nshg, ndof, stepno], nshg * ndof, "double")
        out += block_bytes(_file_order(v).reshape(-1), "double")
    return out


def read_restart(data: bytes, nshg: int, ndof: int = 5):
    R = Reader(data)
    res, lstep = [], 0
    for k, key in enumerate(("solution", "time derivative of solution")):
        h = R.header(key, 3)
        if h is not None and h[0] != 0:
            lstep = h[2]
            q = R.block(h[0] * h[1], "double").reshape(h[1], h[0])[:ndof]
        else:
            q = np.zeros((ndof, nshg))
            if k == 0:
                q[0] = q[4] = 1.0
        res.append(_solver_order(q))
    return res[0], res[1], lstep


# ---- geombc --------------------------------------------------------------------------------

def geombc_bytes(x, interior, nBC, iBCtmp, BCinp, iper, boundary=()) -> bytes:
    """geombc file of the headers readnblk reads.

    ``interior``: list of (ien (neltp, nshl) 1-based, lcsyst); ``boundary``: list of
    (ienb (neltp, nshl) 1-based, iBCB (neltp, 2), BCB (neltp, 6), nenbl, lcsyst).
    """
    x = np.asarray(x, dtype=np.float64)
    numnp = x.shape[0]
    nshg = len(nBC)
    numpbc = len(iBCtmp)
    nen = max([e.shape[1] for e, _ in interior] + [0])
    out = b"# PHASTA Input File Version 2.0\n"
    out += header_bytes("byteorder magic number", [MAGIC], 1, "integer") + block_bytes([MAGIC], "integer")
    counts = [("number of nodes", numnp), ("number of modes", nshg),
              ("number of interior elements", sum(e.shape[0] for e, _ in interior)),
              ("number of boundary elements", sum(b[0].shape[0] for b in boundary)),
              ("maximum number of element nodes", nen), ("number of interior tpblocks", len(interior)),
              ("number of boundary tpblocks", len(boundary)),
              ("number of nodes with Dirichlet BCs", numpbc), ("number of shape functions", nen)]
    for k, v in counts:
        out += header_bytes(k, [v], 0, "integer")
    out += header_bytes("co-ordinates", [numnp, 3], numnp * 3, "double")
    out += block_bytes(x.T.reshape(-1), "double")
    for ien, lcsyst in interior:
        ne, nshl = ien.shape
        key = f"connectivity interior linear {_TOPO[lcsyst]}"
        out += header_bytes(key, [ne, nshl, 1, nshl, 0, 0, lcsyst], ne * nshl, "integer")
        out += block_bytes(np.asarray(ien).T.reshape(-1), "integer")
    out += header_bytes("bc mapping array", [nshg], nshg, "integer") + block_bytes(nBC, "integer")
    out += header_bytes("bc codes array", [numpbc], numpbc, "integer") + block_bytes(iBCtmp, "integer")
    B = np.asarray(BCinp, dtype=np.float64)
    out += header_bytes("boundary condition array", [B.size], B.size, "double")
    out += block_bytes(B.T.reshape(-1), "double")
    out += header_bytes("periodic masters array", [nshg], nshg, "integer") + block_bytes(iper, "integer")
    for ienb, ibcb, bcb, nenbl, lcsyst in boundary:
        ne, nshl = ienb.shape
        topo = _TOPO[lcsyst]
        h = [ne, nshl, 1, nshl, nenbl, nenbl, lcsyst, 6]
        out += header_bytes(f"connectivity boundary linear {topo}", h, ne * nshl, "integer")
        out += block_bytes(np.asarray(ienb).T.reshape(-1), "integer")
        out += header_bytes(f"nbc codes linear {topo}", h, ne * 2, "integer")
        out += block_bytes(np.asarray(ibcb).T.reshape(-1), "integer")
        out += header_bytes(f"nbc values linear {topo}", h, ne * 6, "double")
        out += block_bytes(np.asarray(bcb).T.reshape(-1), "double")
    return out


_TOPO = {1: "tetrahedron", 2: "hexahedron", 3: "wedge", 5: "pyramid"}


def read_geombc(data: bytes, ndof: int = 5):
    R = Reader(data)
    g = {}
    for k in ("number of nodes", "number of modes", "number of interior elements",
              "number of boundary elements", "maximum number of element nodes",
              "number of interior tpblocks", "number of boundary tpblocks",
              "number of nodes with Dirichlet BCs", "number of shape functions"):
        g[k] = R.header(k, 1)[0]
    numnp, nsd = R.header("co-ordinates", 2)
    g["x"] = R.block(numnp * nsd, "double").reshape(nsd, numnp).T
    g["interior"] = []
    for _ in range(g["number of interior tpblocks"]):
        h = R.header("connectivity interior?", 7)
        ne, nshl = h[0], h[3]
        g["interior"].append((h, R.block(ne * nshl, "integer").reshape(nshl, ne).T))
    nshg = R.header("bc mapping array", 1)[0]
    g["nBC"] = R.block(nshg, "integer")
    numpbc = R.header("bc codes array", 1)[0]
    g["iBCtmp"] = R.block(numpbc, "integer")
    size = R.header("boundary condition array", 1)[0]
    B = R.block(size, "double")
    g["BCinp"] = B.reshape(size // numpbc, numpbc).T if numpbc else B
    nshg = R.header("periodic masters array", 1)[0]
    g["iper"] = R.block(nshg, "integer")
    g["boundary"] = []
    nd = ndof + 1
    for _ in range(g["number of boundary tpblocks"]):
        h = R.header("connectivity boundary?", 8)
        ne, nshl, nshlb, nenbl = h[0], h[3], h[4], h[5]
        ienb = R.block(ne * nshl, "integer").reshape(nshl, ne).T
        R.header("nbc codes?", 8)
        codes = R.block(ne * 2, "integer").reshape(2, ne).T
        R.header("nbc values?", 8)
        vals = R.block(ne * nd, "double").reshape(nd, ne).T.copy()
        c = codes[:, 0]
        vals[(c & 1) == 0, 0] = 0.0
        vals[(c & 2) == 0, 1] = 0.0
        vals[(c & 8) == 0, 5] = 0.0
        vals[(c & 4) == 0, 2:5] = 0.0
        bcb = np.zeros((ne, nshlb, nd))
        bcb[:, :nenbl, :] = vals[:, None, :]
        g["boundary"].append((h, ienb, codes, bcb))
    return g


# ---- geniBC / genBC1 -----------------------------------------------------------------------

def genibc(nBC, iBCtmp):
    nBC = np.asarray(nBC)
    iBC = np.zeros(len(nBC), dtype=np.int32)
    if len(iBCtmp):
        m = nBC != 0
        iBC[m] = np.asarray(iBCtmp)[nBC[m] - 1]
    return iBC


def genbc1(BCinp, nBC, iBC, ndof: int = 5):
    """BC (nshg, ndof+1) from BCinp (numpbc, >= ndof+7), following genbc1.f's WHERE order."""
    nBC = np.asarray(nBC)
    N = len(nBC)
    T = np.zeros((N, ndof + 7))
    m = nBC != 0
    if np.asarray(BCinp).size:
        T[m] = np.asarray(BCinp)[nBC[m] - 1, :ndof + 7]
    iBC = np.asarray(iBC)
    BC = np.zeros((N, ndof + 1))
    with np.errstate(divide="ignore", invalid="ignore"):
        for s in range(1, ndof - 4):
            w = (iBC >> (5 + s)) & 1 == 1
            BC[w, 5 + s] = T[w, 11 + s]
        w = iBC & 1 == 1
        BC[w, 0] = T[w, 0]
        w = iBC & 2 == 2
        BC[w, 1] = T[w, 1]
        w = iBC & 4 == 4
        BC[w, 0] = T[w, 2]
        v = (iBC >> 3) & 7

        def c(k):  # 1-based column of BCtmp
            return k - 1

        for case, piv, o1, o2 in ((1, 4, 5, 6), (2, 5, 4, 6), (4, 6, 4, 5)):
            w = v == case
            tmp = T[w, 3] ** 2 + T[w, 4] ** 2 + T[w, 5] ** 2
            BC[w, 2] = tmp * T[w, 6] / T[w, c(piv)]
            BC[w, 3] = T[w, c(o1)] / T[w, c(piv)]
            BC[w, 4] = T[w, c(o2)] / T[w, c(piv)]
        for case, z1, z2 in ((3, 4, 9), (5, 4, 10), (6, 5, 10)):
            w = np.where(v == case)[0]
            for i in w:
                if T[i, c(z1)] == 0 or T[i, c(z2)] == 0:
                    T[i, 3:7], T[i, 7:11] = T[i, 7:11].copy(), T[i, 3:7].copy()
            if not len(w):
                continue
            t = T[w]
            a = np.sqrt(t[:, 3] ** 2 + t[:, 4] ** 2 + t[:, 5] ** 2)
            t[:, 3:6] /= a[:, None]
            t[:, 6] *= a
            b = np.sqrt(t[:, 7] ** 2 + t[:, 8] ** 2 + t[:, 9] ** 2)
            t[:, 7:10] /= b[:, None]
            t[:, 10] *= b
            col = lambda k: t[:, k - 1]  # noqa: E731
            out = BC[w]
            if case == 3:
                t[:, 3] = col(9) * col(4) - col(5) * col(8)
                t[:, 5] = col(9) * col(6) - col(5) * col(10)
                t[:, 6] = col(9) * col(7) - col(5) * col(11)
                out[:, 2], out[:, 3] = col(7) / col(4), col(6) / col(4)
                t[:, 8] = col(4) * col(9)
                t[:, 9] = col(4) * col(10) - col(8) * col(6)
                t[:, 10] = col(4) * col(11) - col(8) * col(7)
                out[:, 4], out[:, 5] = col(11) / col(9), col(10) / col(9)
            elif case == 5:
                t[:, 3] = col(10) * col(4) - col(6) * col(8)
                t[:, 4] = col(10) * col(5) - col(6) * col(9)
                t[:, 6] = col(10) * col(7) - col(6) * col(11)
                out[:, 2], out[:, 3] = col(7) / col(4), col(5) / col(4)
                t[:, 8] = col(4) * col(9) - col(8) * col(5)
                t[:, 9] = col(4) * col(10)
                t[:, 10] = col(4) * col(11) - col(8) * col(7)
                out[:, 4], out[:, 5] = col(11) / col(10), col(9) / col(10)
            else:
                t[:, 3] = col(10) * col(4) - col(6) * col(8)
                t[:, 4] = col(10) * col(5) - col(6) * col(9)
                t[:, 6] = col(10) * col(7) - col(6) * col(11)
                out[:, 2], out[:, 3] = col(7) / col(5), col(4) / col(5)
                t[:, 7] = col(5) * col(8) - col(9) * col(4)
                t[:, 9] = col(5) * col(10)
                t[:, 10] = col(5) * col(11) - col(9) * col(7)
                out[:, 4], out[:, 5] = col(11) / col(10), col(8) / col(10)
            BC[w] = out
            T[w] = t
        w = v == 7
        BC[w, 2] = T[w, 6] * T[w, 3]
        BC[w, 3] = T[w, 6] * T[w, 4]
        BC[w, 4] = T[w, 6] * T[w, 5]
    return BC
