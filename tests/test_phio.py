"""PHASTA file I/O of the GPU path, on the CPU (the library's host-only entry points).

The C++ reader/writer (csrc/phio.cpp, include/phgpu_io.h) is checked against the
oracle's restatement of phastaIO's POSIX format (oracle/phio_oracle.py): files
written by one are read by the other, byte for byte where the format fixes the
bytes (headers, blocks, restart files), with the reader's search rules (case and
blanks ignored, '?' wildcards, comments, skipping and wrapping around, byte-swapped
files), and geniBC/genBC1 against the reference's own Fortran run through the
translator (tests/golden/ref_genbc.npz, bit for bit).  Geombc and restart files of
the benchmark meshes go through a write -> read round trip; checkphasta compares
case directories as the reference tool does.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np
import pytest

from helpers import channel, mixed
from oracle import phio_oracle as O
from phasta_gb300 import _lib as L
from phasta_gb300 import phio

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def _write_mixed_file(path, iotype="binary"):
    rng = np.random.default_rng(7)
    ints = rng.integers(-50, 50, size=17).astype(np.int32)
    dbl = rng.standard_normal(11)
    with phio.PhastaFile(path, "write", iotype) as f:
        f.writestring("# PHASTA Input File Version 2.0\n")
        f.write("byteorder magic number", [362436], [362436], "integer")
        f.writeheader("number of nodes", [4913], 0, "integer")
        f.write("co-ordinates", [11, 1], dbl, "double")
        f.write("connectivity interior linear tetrahedron", [17, 1, 1, 1, 0, 0, 1], ints, "integer")
        f.write("empty block", [0], np.zeros(0), "double")
    return ints, dbl


def _oracle_mixed_bytes(ints, dbl, iotype="binary"):
    out = b"# PHASTA Input File Version 2.0\n"
    out += O.header_bytes("byteorder magic number", [362436], 1, "integer", iotype)
    out += O.block_bytes([362436], "integer", iotype)
    out += O.header_bytes("number of nodes", [4913], 0, "integer", iotype)
    out += O.header_bytes("co-ordinates", [11, 1], 11, "double", iotype) + O.block_bytes(dbl, "double", iotype)
    out += O.header_bytes("connectivity interior linear tetrahedron", [17, 1, 1, 1, 0, 0, 1], 17, "integer", iotype)
    out += O.block_bytes(ints, "integer", iotype)
    out += O.header_bytes("empty block", [0], 0, "double", iotype) + O.block_bytes(np.zeros(0), "double", iotype)
    return out


@pytest.mark.parametrize("iotype", ["binary", "ascii"])
def test_writer_bytes_match_the_format(tmp_path, iotype):
    p = tmp_path / "f.dat"
    ints, dbl = _write_mixed_file(p, iotype)
    assert p.read_bytes() == _oracle_mixed_bytes(ints, dbl, iotype)


def test_reader_search_rules(tmp_path):
    """Comments, blank lines, case and blank insensitivity, '?' wildcards, skipping of
    other blocks and the wrap-around to the start of the file."""
    ints, dbl = _write_mixed_file(tmp_path / "f.dat")
    data = (tmp_path / "f.dat").read_bytes()
    # comments and blank lines between blocks
    data = data.replace(b"number of nodes", b"\n# a comment line\n\nNumber  Of nodes", 1)
    p = tmp_path / "g.dat"
    p.write_bytes(data)
    R = O.Reader(data)
    with phio.PhastaFile(p) as f:
        # out of file order: the search wraps around
        h = f.readheader("connectivity interior?", 7)
        assert list(h) == [17, 1, 1, 1, 0, 0, 1] == R.header("connectivity interior?", 7)
        assert np.array_equal(f.readdatablock("connectivity interior?", 17, "integer"), ints)
        assert np.array_equal(R.block(17, "integer"), ints)
        assert list(f.readheader("numberofnodes", 1)) == [4913] == R.header("numberofnodes", 1)
        assert list(f.readheader("CO-ORDINATES", 2, "double")) == [11, 1] == R.header("CO-ORDINATES", 2)
        assert np.array_equal(f.readdatablock("co-ordinates", 11), dbl)
        assert np.array_equal(R.block(11, "double"), dbl)
        # a key that is only a prefix of the file's key matches (cscompare)
        assert list(f.readheader("connectivity", 1)) == [17] == R.header("connectivity", 1)
        f.readdatablock("connectivity", 17, "integer")
        R.block(17, "integer")
        # more integers asked than the header has: the trailing newline counts as one (0),
        # the third value is left as it was
        assert list(f.readheader("number of nodes", 3)) == [4913, 0, 0]
        assert f.readheader("no such key", 1) is None
        assert R.header("no such key", 1) is None


def test_not_found_leaves_outputs_and_skips_the_block(tmp_path):
    _write_mixed_file(tmp_path / "f.dat")
    lib = L.lib()
    with phio.PhastaFile(tmp_path / "f.dat") as f:
        v = np.full(2, 77, np.int32)
        rc = lib.phgpu_io_readheader(f.fd, b"solution", L.iptr(v), 2, b"double", b"binary")
        assert rc == L.PHGPU_ERR_NOTFOUND and list(v) == [77, 77]
        a = np.full(3, 5.0)
        rc = lib.phgpu_io_readdatablock(f.fd, b"solution", L.dptr(a), 3, b"double", b"binary")
        assert rc == L.PHGPU_ERR_NOTFOUND and list(a) == [5.0] * 3


def test_strict_mode_checks_header_block_pairs(tmp_path):
    lib = L.lib()
    p = tmp_path / "s.dat"
    with phio.PhastaFile(p, "write") as f:
        f.writeheader("alpha", [3], 3, "double")
        # lenient (the reference's default): a mismatched key only warns
        f.writedatablock("beta", np.ones(3))
    assert lib.phgpu_io_togglestrictmode() == 1
    try:
        with phio.PhastaFile(tmp_path / "t.dat", "write") as f:
            f.writeheader("alpha", [3], 3, "double")
            with pytest.raises(phio.PhastaIOError):
                f.writedatablock("beta", np.ones(3))
            f.writeheader("gamma", [3], 3, "double")
            with pytest.raises(phio.PhastaIOError):
                f.writedatablock("gamma", np.ones(2))
    finally:
        assert lib.phgpu_io_togglestrictmode() == 0


def test_byte_swapped_file_is_detected(tmp_path):
    """A file written on a machine of the other byte order: the magic number read back
    differs from 362436 and every later block is swapped (phastaIO.cc:251-256, 1474)."""
    rng = np.random.default_rng(3)
    ints = rng.integers(-1000, 1000, 9).astype(np.int32)
    dbl = rng.standard_normal(5)
    be = b"byteorder magic number : < 5 > 1 \n" + struct.pack(">i", 362436) + b"\n"
    be += b"solution : < 41 > 5 1 0 \n" + dbl.astype(">f8").tobytes() + b"\n"
    be += b"codes : < 37 > 9 \n" + ints.astype(">i4").tobytes() + b"\n"
    p = tmp_path / "be.dat"
    p.write_bytes(be)
    with phio.PhastaFile(p) as f:
        assert list(f.readheader("solution", 3)) == [5, 1, 0]
        assert np.array_equal(f.readdatablock("solution", 5), dbl)
        f.readheader("codes", 1)
        assert np.array_equal(f.readdatablock("codes", 9, "integer"), ints)
    R = O.Reader(be)
    R.header("solution", 3)
    assert np.array_equal(R.block(5, "double"), dbl)


def test_restart_files(tmp_path):
    rng = np.random.default_rng(11)
    nshg = 1234
    y, ac = rng.standard_normal((5, nshg)), rng.standard_normal((5, nshg))
    p = phio.write_restart(tmp_path, 7, y, ac)
    assert p.name == "restart.7.1"
    assert p.read_bytes() == O.restart_bytes(y, ac, 7)
    y2, ac2, lstep = phio.read_restart(tmp_path, 7, nshg)
    assert lstep == 7 and np.array_equal(y2, y) and np.array_equal(ac2, ac)
    yo, aco, so = O.read_restart(p.read_bytes(), nshg)
    assert so == 7 and np.array_equal(yo, y) and np.array_equal(aco, ac)
    # the file holds (p, u, v, w, T): restar's reordering of the solver's (u, v, w, p, T)
    with phio.PhastaFile(p) as f:
        f.readheader("solution", 3)
        q = f.readdatablock("solution", 5 * nshg).reshape(5, nshg)
    assert np.array_equal(q[0], y[3]) and np.array_equal(q[1:4], y[:3]) and np.array_equal(q[4], y[4])
    # rank 2 writes part 3; a wrong nshg is an error, as readnblk's error('restar')
    phio.write_restart(tmp_path, 7, y, ac, rank=2)
    assert (tmp_path / "restart.7.3").exists()
    with pytest.raises(phio.PhastaIOError):
        phio.read_restart(tmp_path, 7, nshg + 1)


def test_restart_defaults_when_fields_are_missing(tmp_path):
    """No time derivative: ac = 0; no solution either: p = T = 1 (readnblk.f:517-558)."""
    nshg = 10
    y = np.arange(5 * nshg, dtype=np.float64).reshape(5, nshg)
    with phio.PhastaFile(tmp_path / "restart.3.1", "write") as f:
        f.write("byteorder magic number", [362436], [362436], "integer")
        f.write("solution", [nshg, 5, 3], O._file_order(y).reshape(-1), "double")
    y2, ac2, lstep = phio.read_restart(tmp_path, 3, nshg)
    assert lstep == 3 and np.array_equal(y2, y) and not ac2.any()
    with phio.PhastaFile(tmp_path / "restart.4.1", "write") as f:
        f.write("byteorder magic number", [362436], [362436], "integer")
    y3, ac3, lstep = phio.read_restart(tmp_path, 4, nshg)
    expect = np.zeros((5, nshg))
    expect[3] = expect[4] = 1.0
    assert lstep == 0 and np.array_equal(y3, expect) and not ac3.any()


def test_genbc_matches_the_reference_fortran():
    d = np.load(GOLDEN / "ref_genbc.npz")
    iBC, BC = phio.boundary_conditions(d["nBC"], d["iBCtmp"], d["BCinp"])
    assert np.array_equal(iBC, d["iBC"])
    assert np.array_equal(BC, d["BC"].T)
    # the oracle's restatement agrees as well
    assert np.array_equal(O.genibc(d["nBC"], d["iBCtmp"]), d["iBC"])
    assert np.array_equal(O.genbc1(d["BCinp"], d["nBC"], d["iBC"]), d["BC"])


def test_genbc_refuses_periodic_rotation():
    nBC = np.array([1, 0], np.int32)
    BCinp = np.zeros((1, 12))
    BCinp[0, 11] = 0.5
    with pytest.raises(phio.PhastaIOError) as e:
        phio.boundary_conditions(nBC, np.array([1024], np.int32), BCinp)
    assert e.value.code == L.PHGPU_ERR_UNSUPPORTED


def _same_case(a, b):
    assert a.nshg == b.nshg
    for k in ("x", "ien", "ienb", "iBCB", "BCB", "iBC", "BC", "iper", "ienh", "ienw"):
        assert np.array_equal(np.asarray(getattr(a, k)), np.asarray(getattr(b, k))), k
    assert a.h == pytest.approx(b.h, rel=1e-12)
    assert [blk.lcsyst for blk in a.bnd] == [blk.lcsyst for blk in b.bnd]
    for x, y in zip(a.bnd, b.bnd):
        for k in ("ien", "iBCB", "BCB"):
            assert np.array_equal(getattr(x, k), getattr(y, k)), (x.lcsyst, k)


@pytest.mark.parametrize("make", [lambda: channel(4, ac_scale=0.05), lambda: mixed(3, 3, (3, 3, 2))],
                         ids=["channel4", "mixed3"])
def test_geombc_round_trip(tmp_path, make):
    case = make()[0]
    path = phio.write_case(case, tmp_path)
    assert path.name == "geombc.dat.1"
    back = phio.read_case(tmp_path)
    _same_case(case, back)
    # the oracle reads the same arrays from the file
    g = O.read_geombc(path.read_bytes())
    assert np.array_equal(g["x"], case.x)
    assert np.array_equal(O.genibc(g["nBC"], g["iBCtmp"]), case.iBC)
    assert np.array_equal(O.genbc1(g["BCinp"], g["nBC"], O.genibc(g["nBC"], g["iBCtmp"])), case.BC.T)
    assert np.array_equal(g["iper"] - 1, case.iper)
    # and a file written by the oracle reads back the same through the library
    interior = [(np.asarray(e) + 1, lc) for e, lc in ((case.ien, 1), (case.ienh, 2), (case.ienw, 3)) if len(e)]
    boundary = [(case.ienb + 1, case.iBCB, case.BCB[:, 0, :], 3, 1)] if case.nbelem else []
    nBC, codes, rows = phio._bcinp(case)
    (tmp_path / "o").mkdir()
    (tmp_path / "o" / "geombc.dat.1").write_bytes(
        O.geombc_bytes(case.x, interior, nBC, codes, rows, case.iper + 1, boundary))
    _same_case(case, phio.read_case(tmp_path / "o"))


@pytest.mark.parametrize("which", ["layered_open", "wedge_channel"])
def test_geombc_round_trip_with_boundary_hexes_and_wedges(tmp_path, which):
    """Boundary blocks of hexes (lcsyst 2) and of wedges with triangle or quadrilateral faces
    (lcsyst 3 with nenbl 3 or 4) through the file: the wedge block's face size selects its
    boundary rule on reading; BC codes and values per element, spread over the face nodes."""
    from helpers import layered, wedgechannel
    case = layered(4, (2, 1, 2), periodic_x=False)[0] if which == "layered_open" else wedgechannel((3, 3, 2))[0]
    rng = np.random.default_rng(9)
    for b in case.bnd:
        n = len(b.ien)
        b.iBCB = np.stack([np.full(n, 3), np.arange(n) % 4], axis=1).astype(np.int32)  # mass flux and pressure set
        vals = np.zeros((n, 6))
        vals[:, :2] = rng.standard_normal((n, 2))
        b.BCB = np.repeat(vals[:, None, :], b.nshlb, axis=1)
    phio.write_case(case, tmp_path)
    back = phio.read_case(tmp_path)
    _same_case(case, back)


def test_geombc_boundary_values_are_masked_by_flux_codes(tmp_path):
    case = channel(3, ac_scale=0.05)[0]
    nb = case.nbelem
    rng = np.random.default_rng(5)
    case.iBCB = np.stack([rng.integers(0, 16, nb), np.ones(nb)], axis=1).astype(np.int32)
    vals = rng.standard_normal((nb, 6))
    case.BCB = np.repeat(vals[:, None, :], 3, axis=1)
    phio.write_case(case, tmp_path)
    back = phio.read_case(tmp_path)
    c = case.iBCB[:, 0]
    expect = vals.copy()
    expect[(c & 1) == 0, 0] = 0
    expect[(c & 2) == 0, 1] = 0
    expect[(c & 8) == 0, 5] = 0
    expect[(c & 4) == 0, 2:5] = 0
    assert np.array_equal(back.BCB, np.repeat(expect[:, None, :], 3, axis=1))


def test_checkphasta(tmp_path):
    rng = np.random.default_rng(2)
    nshg = 50
    left, right = tmp_path / "l", tmp_path / "r"
    left.mkdir()
    right.mkdir()
    y = rng.standard_normal((5, nshg))
    for step in (0, 5, 10):
        phio.write_restart(left, step, y + step, y)
    for step in (5, 10, 15):
        z = y + step
        if step == 10:
            z = z.copy()
            z[2, 7] += 3e-6
        phio.write_restart(right, step, z, y)
    m, n, ok = phio.checkphasta(left, right, 1e-5)
    assert n == 2 and ok and m == pytest.approx(3e-6, rel=1e-6)
    m, n, ok = phio.checkphasta(left, right, 1e-6)
    assert not ok
