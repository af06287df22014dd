"""CPU tests of the oracle: pinned tables, invariants with exact answers, LU, BCs."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from helpers import channel, rel, vortex
from oracle import pyoracle
from phasta_gb300 import mesh

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_tables_match_reference_c_sources():
    """symtet.c/symtri.c/TetShapeAndDrv of the reference, tabulated by make_tables.py."""
    g = json.loads((GOLDEN / "tet_tables.json").read_text())
    t = pyoracle.tet_tables()
    for k in ("shp", "shgl", "Qwt", "shpb", "shglb", "Qwtb"):
        assert np.array_equal(np.array(g[k]), t[k]), k


@pytest.mark.parametrize("iDC", [0, 1, 2, 3])
def test_uniform_freestream_has_zero_residual(iDC):
    case, p, y, ac = channel(8, sigma=0.0, iDC=iDC)
    o = pyoracle.Oracle(case, p)
    res, rmes, bd = o.ElmMFG(y, ac)
    # flux magnitudes are O(p) ~ 8: a free stream is an exact solution (the DC factor of
    # zero gradients and residuals is zero: raLS = rTLS = 0, gnorm = 1/epsM)
    assert np.abs(res).max() < 1e-12
    assert np.isfinite(bd).all()


def test_discontinuity_capturing_leaves_bdiag():
    """The matrix-free block diagonal has no DC term (e3bdg.f takes no DC stiffness); the
    residual does."""
    case, p, y, ac = channel(6, sigma=0.05, ac_scale=0.05)
    r0, _m0, b0 = pyoracle.Oracle(case, p).ElmMFG(y, ac)
    for iDC in (1, 2, 3):
        r, _m, b = pyoracle.Oracle(case, dict(p, iDC=iDC)).ElmMFG(y, ac)
        assert np.array_equal(b, b0)
        assert np.linalg.norm(r - r0) > 1e-8 * np.linalg.norm(r0)


def test_periodic_vortex_runs_and_is_finite():
    case, p, y, ac = vortex(6)
    o = pyoracle.Oracle(case, p)
    res, rmes, bd = o.ElmMFG(y, ac)
    assert case.nbelem == 0
    assert np.isfinite(res).all() and np.linalg.norm(res) > 0


def _elem_inputs(seed=3):
    g = np.random.default_rng(seed)
    fs = mesh.freestream(0.3)
    xl = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 1.0, 0.1], [0.1, 0.2, 1.0]]) * 0.1
    # orientation used by the reference: det[x1-x4, x2-x4, x3-x4] > 0
    if np.linalg.det(np.stack([xl[0] - xl[3], xl[1] - xl[3], xl[2] - xl[3]])) < 0:
        xl[[0, 1]] = xl[[1, 0]]
    base = np.array([fs["p"], fs["u"], 0.0, 0.0, fs["T"]])
    scale = np.array([fs["p"], 1.0, 1.0, 1.0, fs["T"]])
    yl = base + 0.02 * scale * g.standard_normal((4, 5))
    acl = 0.1 * scale * g.standard_normal((4, 5))
    return xl, yl, acl


def _params():
    case, p, _, _ = channel(4)
    return p


def test_element_node_permutation_invariance():
    """An even permutation of the local nodes permutes the element contributions."""
    p = _params()
    xl, yl, acl = _elem_inputs()
    rl, rml, bd = pyoracle.e3(p, yl, yl, acl, xl, ires=3, iprec=1)
    perm = [1, 2, 0, 3]  # cyclic on the first three nodes keeps the orientation
    rl2, rml2, bd2 = pyoracle.e3(p, yl[perm], yl[perm], acl[perm], xl[perm], ires=3, iprec=1)
    assert rel(rl2, rl[perm]) < 1e-12
    assert rel(rml2, rml[perm]) < 1e-12
    assert rel(bd2, bd[perm]) < 1e-12


def test_element_rotation_equivariance():
    """Rotating the element and the velocities by 90 deg about z rotates the momentum rows."""
    p = _params()
    xl, yl, acl = _elem_inputs(5)
    Q = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    rot = lambda v: np.concatenate([v[:, :1], v[:, 1:4] @ Q.T, v[:, 4:]], axis=1)  # noqa: E731
    rl, rml, bd = pyoracle.e3(p, yl, yl, acl, xl, ires=3, iprec=1)
    rl2, rml2, bd2 = pyoracle.e3(p, rot(yl), rot(yl), rot(acl), xl @ Q.T, ires=3, iprec=1)
    assert rel(rl2, rot(rl)) < 1e-11
    assert rel(rml2, rot(rml)) < 1e-11
    T5 = np.eye(5)
    T5[1:4, 1:4] = Q
    bd_rot = np.einsum("ij,ajk,lk->ail", T5, bd, T5)
    assert rel(bd2, bd_rot) < 1e-11


def test_modified_residual_matches_residual_time_terms():
    """ires=2 with yl = ycl equals the modified residual of ires=3 (rmes used by Au1MFG)."""
    p = _params()
    xl, yl, acl = _elem_inputs(7)
    _, rml3, _ = pyoracle.e3(p, yl, yl, acl, xl, ires=3, iprec=0)
    _, rml2, _ = pyoracle.e3(p, yl, yl, acl, xl, ires=2, iprec=0)
    assert np.array_equal(rml2, rml3)


def _blocks_to_ref(blocks):
    return np.ascontiguousarray(np.transpose(blocks, (2, 1, 0))).reshape(-1)  # (nshg,5,5) column-major


def test_i3lu_factor_solve_product():
    """i3lu.f solves exactly when its skipped U(4,5) update term vanishes."""
    case, p, y, ac = channel(4)
    o = pyoracle.Oracle(case, p)
    g = np.random.default_rng(1)
    N = case.nshg
    blocks = g.standard_normal((N, 5, 5)) + 6.0 * np.eye(5)
    blocks[:, 3, :3] = 0.0  # L(4,1:3) = 0, so U(4,5) needs no update
    r = g.standard_normal((5, N))
    lu, _ = o.i3LU(_blocks_to_ref(blocks), None, 0)
    _, z = o.i3LU(lu, r.reshape(-1).copy(), 1)
    _, x = o.i3LU(lu, z, 2)
    ref = np.linalg.solve(blocks, r.T[:, :, None])[:, :, 0].T
    assert rel(x.reshape(5, N), ref) < 1e-13
    _, ux = o.i3LU(lu, x.copy(), 3)
    _, back = o.i3LU(lu, ux, 2)
    assert rel(back, x) < 1e-13


def test_i3lu_leaves_u45_unupdated_as_the_reference():
    """i3lu.f:41-97 updates every upper entry of rows 2-5 except U(4,5)."""
    case, p, y, ac = channel(4)
    o = pyoracle.Oracle(case, p)
    N = case.nshg
    g = np.random.default_rng(4)
    blocks = g.standard_normal((N, 5, 5)) + 6.0 * np.eye(5)
    lu, _ = o.i3LU(_blocks_to_ref(blocks), None, 0)
    F = lu.reshape(5, 5, N).transpose(2, 1, 0)  # F[n, i, j]
    assert np.array_equal(F[:, 3, 4], blocks[:, 3, 4])
    Lm = np.tril(F, -1) + np.eye(5)
    Um = np.triu(F, 1) + np.einsum("nii->ni", 1.0 / F)[:, :, None] * np.eye(5)
    prod = Lm @ Um
    # every entry but (4,5) reproduces A; (4,5) misses sum_m L(4,m) U(m,5)
    mask = np.ones((5, 5), bool)
    mask[3, 4] = False
    assert np.abs((prod - blocks)[:, mask]).max() < 1e-12
    miss = np.einsum("nm,nm->n", Lm[:, 3, :3], Um[:, :3, 4])
    assert np.allclose(prod[:, 3, 4] - blocks[:, 3, 4], miss, atol=1e-12)


def test_bc3res_zeroes_constrained_rows_and_sums_periodic():
    case, p, y, ac = channel(4)
    o = pyoracle.Oracle(case, p)
    g = np.random.default_rng(2)
    r = g.standard_normal(5 * case.nshg)
    out = o.bc3Res(y, r).reshape(5, -1)
    r = r.reshape(5, -1)
    ib = case.iBC
    slave = (ib >> 10) & 1 == 1
    assert np.all(out[:, slave] == 0.0)
    inflow = ((ib >> 3) & 7) == 7
    assert np.all(out[1:5, inflow] == 0.0)
    # total of the unconstrained continuity row is conserved by the periodic sum
    free = ~inflow
    assert abs(out[0].sum() - r[0].sum()) < 1e-10 * np.abs(r[0]).sum() + 1e-12 or np.any(~free)


def test_gmres_converges_and_newton_reduces_residual():
    case, p, y, ac = channel(8, Kspace=10, etol=1e-3, minIters=1)
    o = pyoracle.Oracle(case, p)
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    y1, ac1, st, Dy = o.newton(y, ac, y, ac)
    r1 = np.linalg.norm(o.ElmRes(y1, ac1))
    assert st.echeck <= 1e-3 * st.unorm0
    assert r1 < 0.05 * r0


def test_threaded_grouped_sweep_matches_sequential():
    case, p, y, ac = channel(8)
    a = pyoracle.Oracle(case, p, nthreads=1)
    b = pyoracle.Oracle(case, p, nthreads=4)
    ra, ma, ba = a.ElmMFG(y, ac)
    rb, mb, bb = b.ElmMFG(y, ac)
    assert rel(rb, ra) < 1e-13 and rel(mb, ma) < 1e-13 and rel(bb, ba) < 1e-13


def test_mesh_orientation_normals_and_periodicity():
    case, _ = mesh.channel_case(6)
    x = case.x
    e = case.ien
    det = np.einsum("ij,ij->i", x[e[:, 0]] - x[e[:, 3]], np.cross(x[e[:, 1]] - x[e[:, 3]], x[e[:, 2]] - x[e[:, 3]]))
    assert np.all(det > 0)
    assert case.nelem == 6 * 6 ** 3
    b = case.ienb
    n = np.cross(x[b[:, 1]] - x[b[:, 0]], x[b[:, 2]] - x[b[:, 0]])
    inward = x[b[:, 3]] - x[b[:, 0]]
    assert np.all(np.einsum("ij,ij->i", n, inward) < 0)  # face normal points out of the element
    assert np.all(case.iper[case.iper] == case.iper)     # masters are not slaves
    assert case.nbelem == 2 * 2 * 6 * 6


def test_oracle_groups_are_conflict_free():
    case, p, y, ac = channel(6)
    o = pyoracle.Oracle(case, p, nthreads=2, grouped=True)
    ien = o._ien.reshape(-1, 4)
    for gI in range(len(o._grp) - 1):
        b0, b1 = o._grp[gI], o._grp[gI + 1]
        e0, e1 = o._blk[b0], o._blk[b1]
        nodes = ien[e0:e1].reshape(-1)
        assert len(np.unique(nodes)) == len(nodes)


@pytest.mark.parametrize("code", [0, 1])
def test_yshuffle_roundtrip(code):
    L = pyoracle.lib()
    import ctypes as C
    N = 7
    r = np.arange(5 * N, dtype=np.float64)
    a = r.copy()
    L.or_yshuffle(N, a.ctypes.data_as(C.POINTER(C.c_double)), code)
    L.or_yshuffle(N, a.ctypes.data_as(C.POINTER(C.c_double)), 1 - code)
    assert np.array_equal(a, r)


def test_hex_and_wedge_tables_match_reference_c_sources():
    """Oracle restatement of symhex.c/symwdg.c and the hex/wedge shapes vs tests/golden/topo_tables.json."""
    import json
    d = json.loads((Path(__file__).resolve().parent / "golden" / "topo_tables.json").read_text())
    for name, lcsyst in (("hex", 2), ("wedge", 3)):
        t = pyoracle.topo_tables(lcsyst)
        for k in ("shp", "shgl", "Qwt"):
            assert np.array_equal(t[k], np.array(d[name][k])), (name, k)


def test_boundary_hex_and_wedge_tables_match_reference_c_sources():
    """Oracle restatement of the boundary rules (symquad.c, symtri.c reordered, symquadw.c) and shapes
    at their points vs tests/golden/topo_tables.json, and the face nodes of getbnodes."""
    import json
    d = json.loads((Path(__file__).resolve().parent / "golden" / "topo_tables.json").read_text())
    for name, lcsyst, lnode in (("hex_quad_b", 2, [0, 1, 2, 3]), ("wedge_tri_b", 3, [0, 1, 2]),
                                ("wedge_quad_b", 4, [0, 3, 4, 1])):
        t = pyoracle.btopo_tables(lcsyst)
        for k in ("shpb", "shglb", "Qwtb"):
            assert np.array_equal(t[k], np.array(d[name][k])), (name, k)
        assert t["lnode"].tolist() == lnode
        # the face nodes carry the whole shape at every boundary point
        assert np.allclose(t["shpb"][:, lnode].sum(axis=1), 1.0, rtol=0, atol=1e-14)


@pytest.mark.parametrize("which", ["hex", "wedge"])
def test_boundary_faces_integrate_to_the_face_area(which):
    """A uniform pressure, zero velocity, no viscosity: each boundary face adds p n dA to the momentum
    residual, so the x-momentum over the inflow and outflow faces sums to -p A and +p A."""
    from phasta_gb300 import mesh
    from phasta_gb300.solver import make_params
    case = (mesh.hex_box(3, periodic=(False, True, True)) if which == "hex"
            else mesh.wedge_box(3, periodic=(False, True, False)))
    p = make_params(0.0, 1.0, navier=0)
    y = np.zeros(5 * case.nshg)
    y[3 * case.nshg:4 * case.nshg] = 2.5       # p
    y[4 * case.nshg:] = 300.0                  # T
    o = pyoracle.Oracle(case, p)
    import ctypes as C
    res = np.zeros(5 * case.nshg)
    o.L.or_elmres(C.byref(o.c), C.byref(o.m), pyoracle._d(y), pyoracle._d(np.zeros_like(y)), pyoracle._d(res), 0)
    import dataclasses
    interior = pyoracle.Oracle(dataclasses.replace(case, bnd=[]), p)
    res0 = np.zeros(5 * case.nshg)
    o.L.or_elmres(C.byref(interior.c), C.byref(interior.m), pyoracle._d(y), pyoracle._d(np.zeros_like(y)),
                  pyoracle._d(res0), 0)
    fx = (res - res0).reshape(5, -1)[1]       # x-momentum (local dof 2 = u-row) of the faces
    x = case.x[:, 0]
    assert abs(fx[np.isclose(x, 0.0)].sum() + 2.5) < 1e-12
    assert abs(fx[np.isclose(x, 1.0)].sum() - 2.5) < 1e-12
    if which == "wedge":  # the triangle faces (lcsyst 3) on z = 0 and z = 1
        fz = (res - res0).reshape(5, -1)[3]
        z = case.x[:, 2]
        assert abs(fz[np.isclose(z, 0.0)].sum() + 2.5) < 1e-12
        assert abs(fz[np.isclose(z, 1.0)].sum() - 2.5) < 1e-12
