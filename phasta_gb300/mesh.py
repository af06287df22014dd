"""Synthetic meshes, boundary conditions and states of the benchmark cases.

The reference reads partitioned meshes written by its preprocessor; the
benchmark cases here are generated in process with the same data model
(``x(nshg,3)``, tet connectivity, boundary tets with the boundary face first,
``iBC``/``BC``/``iper`` and ``iBCB``/``BCB``):

* a box of n^3 hexahedra, each split into 6 tets along its main diagonal
  (Kuhn/Freudenthal split; conforming across hexes and across periodic
  faces), nodes (n+1)^3 with the periodic slaves stored as in the reference;
* periodic directions identify the last node layer with the first
  (``iper`` points at the ultimate master, ``iBC`` bit 10 marks slaves);
* an inflow face at x = x0 with Dirichlet velocity and temperature
  (iBC bits 1, 3, 4, 5) and natural (flux-computed) boundary faces at x = x0
  and x = x1 (``iBCB`` = 0);
* states: uniform flow along x at a Mach number plus seeded Gaussian noise,
  or the decaying-vortex field of the 42.5M-tet case.

Tet node order follows the reference's convention: det(dx/dxi) > 0 with
N1..N3 = barycentric coordinates 1..3 and N4 = 1 - N1 - N2 - N3, so the
right-handed normal of face (1,2,3) points out of the element (e3bvar.f:161-171).
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

# gas properties of the reference (common.f:101-108, input.f:164-182)
RH = 8.31441
MSH = (2.8e-2, 3.2e-2)
XN2, XO2 = 0.79, 0.21
GAMMA, GAMMA1 = 1.4, 0.4


def rgas() -> float:
    rs1, rs2 = RH / MSH[0], RH / MSH[1]
    return 1.0 / (XN2 / rs1 + XO2 / rs2)


@dataclass
class BndBlock:
    """A block of boundary hexes or wedges (the reference's boundary element blocks of lcsyst
    2, 3 and 4, genbkb.f): the whole element in its local node order with the boundary face
    where the reference's boundary routines look for it (hex: the zeta = -1 face, nodes 1-4;
    wedge, lcsyst 3: the zeta = -1 triangle, nodes 1-3; wedge, lcsyst 4: the s = 0 quadrilateral,
    nodes 1, 4, 5, 2 as getbnodes lists them, hierarchic.f:161-164), its BC codes and values per
    face node in getbnodes' order."""
    lcsyst: int              # 2 hex/quad face, 3 wedge/triangle face, 4 wedge/quad face
    ien: np.ndarray          # (n, nshl) int32
    iBCB: np.ndarray         # (n, 2) int32
    BCB: np.ndarray          # (n, nshlb, 6) float64

    @property
    def nshl(self) -> int:
        return 8 if self.lcsyst == 2 else 6

    @property
    def nshlb(self) -> int:
        return 3 if self.lcsyst == 3 else 4


def bnd_block(lcsyst: int, ien) -> BndBlock:
    ien = np.ascontiguousarray(ien, dtype=np.int32)
    nb = 3 if lcsyst == 3 else 4
    return BndBlock(lcsyst, ien, np.zeros((ien.shape[0], 2), np.int32), np.zeros((ien.shape[0], nb, 6)))


@dataclass
class Case:
    """A mesh with its boundary conditions (0-based, reference layouts)."""
    nshg: int
    x: np.ndarray            # (nshg, 3) float64, stored column-major as x(nshg,3) -> x.T contiguous
    ien: np.ndarray          # (nelem, 4) int32
    ienb: np.ndarray         # (nbelem, 4) int32, boundary face first
    iBCB: np.ndarray         # (nbelem, 2) int32
    BCB: np.ndarray          # (nbelem, 3, 6) float64
    iBC: np.ndarray          # (nshg,) int32
    BC: np.ndarray           # (6, nshg) float64  == BC(nshg,6) column-major
    iper: np.ndarray         # (nshg,) int32
    h: float                 # smallest edge
    meta: dict = field(default_factory=dict)
    # further interior blocks (linear hexes and wedges, the reference's lcsyst 2 and 3)
    ienh: np.ndarray = field(default_factory=lambda: np.zeros((0, 8), np.int32))
    ienw: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.int32))
    # boundary hexes and wedges, one block per boundary element topology
    bnd: list = field(default_factory=list)

    @property
    def nhex(self) -> int:
        return int(self.ienh.shape[0])

    @property
    def nwedge(self) -> int:
        return int(self.ienw.shape[0])

    @property
    def nelem(self) -> int:
        return int(self.ien.shape[0])

    @property
    def nbelem(self) -> int:
        return int(self.ienb.shape[0])

    def x_ref(self) -> np.ndarray:
        """x(nshg,3) in the reference's column-major layout, as a flat array."""
        return np.ascontiguousarray(self.x.T).reshape(-1)


def _kuhn_tets(n: tuple[int, int, int]) -> np.ndarray:
    nx, ny, nz = n
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ii, jj, kk = (a.reshape(-1) for a in (ii, jj, kk))

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    tets = []
    for perm in itertools.permutations(range(3)):
        off = np.zeros(3, dtype=np.int64)
        verts = [nid(ii, jj, kk)]
        for ax in perm:
            off[ax] += 1
            verts.append(nid(ii + off[0], jj + off[1], kk + off[2]))
        tets.append(np.stack(verts, axis=1))
    # interleave so the 6 tets of one hex are consecutive (spatial locality)
    return np.stack(tets, axis=1).reshape(-1, 4)


def _orient(ien: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Reorder each tet so that det[x1-x4, x2-x4, x3-x4] > 0."""
    a, b, c, d = (x[ien[:, k]] for k in range(4))
    det = np.einsum("ij,ij->i", a - d, np.cross(b - d, c - d))
    out = ien.copy()
    neg = det < 0
    out[neg, 0], out[neg, 1] = ien[neg, 1], ien[neg, 0]
    return out


def box(n: int | tuple[int, int, int], lengths=(1.0, 1.0, 1.0), periodic=(False, True, True),
        inflow=None, boundary_faces=True) -> Case:
    """n^3 hexes x 6 tets on [0,Lx]x[0,Ly]x[0,Lz].

    ``inflow``: dict(T=..., u=(u,v,w)) for a Dirichlet inflow at x = 0, or None.
    Non-periodic x faces get boundary tets with natural (computed) fluxes.
    """
    if isinstance(n, int):
        n = (n, n, n)
    nx, ny, nz = n
    npts = (nx + 1, ny + 1, nz + 1)
    nshg = npts[0] * npts[1] * npts[2]
    gx = [np.linspace(0.0, lengths[d], npts[d]) for d in range(3)]
    X, Y, Z = np.meshgrid(*gx, indexing="ij")
    # node id = i + (nx+1)*(j + (ny+1)*k): store in that order
    x = np.stack([X.transpose(2, 1, 0).reshape(-1), Y.transpose(2, 1, 0).reshape(-1),
                  Z.transpose(2, 1, 0).reshape(-1)], axis=1).astype(np.float64)
    ien = _orient(_kuhn_tets(n), x).astype(np.int32)

    idx = np.arange(nshg)
    i = idx % npts[0]
    j = (idx // npts[0]) % npts[1]
    k = idx // (npts[0] * npts[1])
    mi, mj, mk = i.copy(), j.copy(), k.copy()
    if periodic[0]:
        mi[i == nx] = 0
    if periodic[1]:
        mj[j == ny] = 0
    if periodic[2]:
        mk[k == nz] = 0
    iper = (mi + npts[0] * (mj + npts[1] * mk)).astype(np.int32)
    iBC = np.zeros(nshg, dtype=np.int32)
    iBC[iper != idx] |= 1 << 10
    BC = np.zeros((6, nshg), dtype=np.float64)
    if not periodic[0]:
        _inflow(x, iBC, BC, inflow)
    ienb = _tet_x_faces(x, ien, lengths[0]) if boundary_faces and not periodic[0] else np.zeros((0, 4), np.int32)
    nb = ienb.shape[0]
    h = min(lengths[d] / n[d] for d in range(3))
    return Case(nshg=nshg, x=x, ien=ien, ienb=ienb, iBCB=np.zeros((nb, 2), np.int32),
                BCB=np.zeros((nb, 3, 6), np.float64), iBC=iBC, BC=BC, iper=iper, h=h,
                meta={"n": n, "lengths": lengths, "periodic": periodic})


def _inflow(x, iBC, BC, inflow):
    """Dirichlet velocity and temperature (iBC bits 1, 3, 4, 5) on the x = 0 nodes."""
    if inflow is None:
        return
    m = np.isclose(x[:, 0], 0.0)
    iBC[m] |= (1 << 1) | (7 << 3)
    BC[1, m] = inflow["T"]
    BC[2, m], BC[3, m], BC[4, m] = inflow["u"]


def _tet_x_faces(x, ien, lx):
    """Boundary tets of the x = 0 and x = lx planes, face nodes first (orientation swaps nodes
    0/1 only, so the face stays first)."""
    if ien.shape[0] == 0:
        return np.zeros((0, 4), np.int32)
    xs = x[:, 0]
    blist = []
    for plane in (0.0, lx):
        on = np.isclose(xs[ien], plane)
        sel = np.where(on.sum(axis=1) == 3)[0]
        for e in sel:
            face = [ien[e, a] for a in range(4) if on[e, a]]
            inner = [ien[e, a] for a in range(4) if not on[e, a]]
            blist.append(face + inner)
    if not blist:
        return np.zeros((0, 4), np.int32)
    return _orient(np.array(blist, dtype=np.int64), x).astype(np.int32)


def _hex_x_faces(nid, nx, j, k):
    """Boundary hexes of the cells (0, j, k) and (nx-1, j, k): each a right-handed hex whose
    zeta = -1 face lies on x = 0 (xi, eta, zeta along +y, +z, +x) or on x = lx (xi, eta, zeta
    along +z, +y, -x), so -(v1 x v2) of face nodes 1-3 is the outward normal (e3bvar.f:174-176)."""
    lo = [nid(0, j + b, k + c) for b, c in ((0, 0), (1, 0), (1, 1), (0, 1))]
    lo += [nid(1, j + b, k + c) for b, c in ((0, 0), (1, 0), (1, 1), (0, 1))]
    hi = [nid(nx, j + b, k + c) for c, b in ((0, 0), (1, 0), (1, 1), (0, 1))]
    hi += [nid(nx - 1, j + b, k + c) for c, b in ((0, 0), (1, 0), (1, 1), (0, 1))]
    return np.concatenate([np.stack(lo, axis=1), np.stack(hi, axis=1)])


def _wedge_x_faces(nid, nx, j, k):
    """Boundary prisms (triangles in the xy planes, the x = y diagonal) of the cells (0, j, k) and
    (nx-1, j, k), each with its x-plane quadrilateral as the s = 0 face (nodes 1, 2, 4, 5): the
    triangle turned cyclically so that its edge 1-2 lies on the plane; dx/dr x dx/dzeta then points
    out of the domain (e3bvar.f:160-164)."""
    lo = [(0, 1), (0, 0), (1, 1)]   # the cell's (0,0),(1,1),(0,1) prism turned
    hi = [(1, 0), (1, 1), (0, 0)]   # the cell's (0,0),(1,0),(1,1) prism turned
    a = [nid(0 + p, j + q, k) for p, q in lo] + [nid(0 + p, j + q, k + 1) for p, q in lo]
    b = [nid(nx - 1 + p, j + q, k) for p, q in hi] + [nid(nx - 1 + p, j + q, k + 1) for p, q in hi]
    return np.concatenate([np.stack(a, axis=1), np.stack(b, axis=1)])


def _grid(n, lengths, periodic):
    """Nodes of an (n+1)^3 lattice (slaves of periodic faces stored, as in the reference)."""
    nx, ny, nz = n
    npts = (nx + 1, ny + 1, nz + 1)
    nshg = npts[0] * npts[1] * npts[2]
    gx = [np.linspace(0.0, lengths[d], npts[d]) for d in range(3)]
    X, Y, Z = np.meshgrid(*gx, indexing="ij")
    x = np.stack([X.transpose(2, 1, 0).reshape(-1), Y.transpose(2, 1, 0).reshape(-1),
                  Z.transpose(2, 1, 0).reshape(-1)], axis=1).astype(np.float64)
    idx = np.arange(nshg)
    i = idx % npts[0]
    j = (idx // npts[0]) % npts[1]
    k = idx // (npts[0] * npts[1])
    mi, mj, mk = i.copy(), j.copy(), k.copy()
    for d, (m, c, nd) in enumerate(((mi, i, nx), (mj, j, ny), (mk, k, nz))):
        if periodic[d]:
            m[c == nd] = 0
    iper = (mi + npts[0] * (mj + npts[1] * mk)).astype(np.int32)
    iBC = np.zeros(nshg, dtype=np.int32)
    iBC[iper != idx] |= 1 << 10
    return x, iper, iBC, (lambda a, b, c: a + npts[0] * (b + npts[1] * c))


def hex_box(n, lengths=(1.0, 1.0, 1.0), periodic=(True, True, True), inflow=None) -> Case:
    """Box of n^3 linear hexes, periodic in y and z and, by default, in x.

    Local node order of the reference's hex (HexShapeAndDrv in newshape.cc): parent
    (xi, eta, zeta) corners (-,-,-), (+,-,-), (+,+,-), (-,+,-), then the same at zeta = +1;
    xi, eta, zeta run along x, y, z.  With x not periodic the x = 0 and x = lx faces are
    boundary hexes (lcsyst 2), natural fluxes, and ``inflow`` = dict(T=..., u=(u,v,w)) makes
    x = 0 a Dirichlet inflow."""
    if isinstance(n, int):
        n = (n, n, n)
    x, iper, iBC, nid = _grid(n, lengths, periodic)
    ii, jj, kk = (a.reshape(-1) for a in np.meshgrid(*(np.arange(m) for m in n), indexing="ij"))
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    ienh = np.stack([nid(ii + a, jj + b, kk + c) for a, b, c in corners], axis=1).astype(np.int32)
    h = min(lengths[d] / n[d] for d in range(3))
    BC = np.zeros((6, x.shape[0]))
    bnd = []
    if not periodic[0]:
        _inflow(x, iBC, BC, inflow)
        j2, k2 = (a.reshape(-1) for a in np.meshgrid(np.arange(n[1]), np.arange(n[2]), indexing="ij"))
        bnd.append(bnd_block(2, _hex_x_faces(nid, n[0], j2, k2)))
    return Case(nshg=x.shape[0], x=x, ien=np.zeros((0, 4), np.int32), ienb=np.zeros((0, 4), np.int32),
                iBCB=np.zeros((0, 2), np.int32), BCB=np.zeros((0, 3, 6)), iBC=iBC,
                BC=BC, iper=iper, h=h, ienh=ienh, bnd=bnd,
                meta={"n": n, "lengths": lengths, "periodic": tuple(periodic)})


def wedge_box(n, lengths=(1.0, 1.0, 1.0), periodic=(True, True, True), inflow=None) -> Case:
    """Box of n^3 cubes, each split along its x = y diagonal into two prisms with triangles in
    the xy planes; periodic in y and, by default, in x and z.

    Local node order of the reference's wedge (WedgeShapeAndDrv): the triangle at
    zeta = -1 with parent (r, s) = (0, 0), (1, 0), (0, 1), then the triangle at zeta = +1.
    With x not periodic the x-plane faces are boundary prisms with a quadrilateral face
    (lcsyst 4); with z not periodic the z-plane faces are boundary prisms with a triangle face
    (lcsyst 3; at z = lz the prism is listed from its top triangle down, the triangle reversed,
    so that the face is its zeta = -1 triangle)."""
    if isinstance(n, int):
        n = (n, n, n)
    x, iper, iBC, nid = _grid(n, lengths, periodic)
    ii, jj, kk = (a.reshape(-1) for a in np.meshgrid(*(np.arange(m) for m in n), indexing="ij"))
    tris = ([(0, 0), (1, 0), (1, 1)], [(0, 0), (1, 1), (0, 1)])  # counter-clockwise seen from +z
    prisms = []
    for tri in tris:
        bot = [nid(ii + a, jj + b, kk) for a, b in tri]
        top = [nid(ii + a, jj + b, kk + 1) for a, b in tri]
        prisms.append(np.stack(bot + top, axis=1))
    ienw = np.stack(prisms, axis=1).reshape(-1, 6).astype(np.int32)
    h = min(lengths[d] / n[d] for d in range(3))
    BC = np.zeros((6, x.shape[0]))
    bnd = []
    if not periodic[2]:
        i2, j2 = (a.reshape(-1) for a in np.meshgrid(np.arange(n[0]), np.arange(n[1]), indexing="ij"))
        faces = []
        for tri in tris:
            faces.append(np.stack([nid(i2 + a, j2 + b, 0) for a, b in tri] +
                                  [nid(i2 + a, j2 + b, 1) for a, b in tri], axis=1))
            rev = [tri[0], tri[2], tri[1]]
            faces.append(np.stack([nid(i2 + a, j2 + b, n[2]) for a, b in rev] +
                                  [nid(i2 + a, j2 + b, n[2] - 1) for a, b in rev], axis=1))
        bnd.append(bnd_block(3, np.concatenate(faces)))
    if not periodic[0]:
        _inflow(x, iBC, BC, inflow)
        j2, k2 = (a.reshape(-1) for a in np.meshgrid(np.arange(n[1]), np.arange(n[2]), indexing="ij"))
        bnd.append(bnd_block(4, _wedge_x_faces(nid, n[0], j2, k2)))
    return Case(nshg=x.shape[0], x=x, ien=np.zeros((0, 4), np.int32), ienb=np.zeros((0, 4), np.int32),
                iBCB=np.zeros((0, 2), np.int32), BCB=np.zeros((0, 3, 6)), iBC=iBC,
                BC=BC, iper=iper, h=h, ienw=ienw, bnd=bnd,
                meta={"n": n, "lengths": lengths, "periodic": tuple(periodic)})


def layered(nxy: int, n_hex: int, n_wedge: int, n_tet: int, lengths=(1.0, 1.0, 1.0), periodic_x: bool = True,
            inflow=None) -> Case:
    """One connected, fully periodic box of nxy x nxy x (n_hex + n_wedge + n_tet) cells whose z
    layers are, from z = 0 up, hexes, then prisms (two per cell, triangles in the xy planes,
    the x = y diagonal), then Kuhn tets (six per cell).  Neighbouring layers share their
    interface nodes: the prisms' top triangles are faces of the tets above (the Kuhn split cuts
    the horizontal cell faces along the same diagonal), the hexes' top quads carry the prisms'
    bottom triangles, and the periodic wrap in z joins the tets' top to the hexes' bottom.
    Node ids follow one (nxy+1)^2 (nz+1) lattice, periodic slaves stored.  With ``periodic_x``
    False the x = 0 and x = lx planes are boundaries of all three layers: boundary tets
    (triangle faces), boundary hexes (lcsyst 2) and boundary prisms with a quadrilateral face
    (lcsyst 4), natural fluxes, and ``inflow`` makes x = 0 a Dirichlet inflow."""
    nz = n_hex + n_wedge + n_tet
    n = (nxy, nxy, nz)
    x, iper, iBC, nid = _grid(n, lengths, (periodic_x, True, True))
    ii, jj = (a.reshape(-1) for a in np.meshgrid(np.arange(nxy), np.arange(nxy), indexing="ij"))
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    hexes, prisms, tets = [], [], []
    tris = ([(0, 0), (1, 0), (1, 1)], [(0, 0), (1, 1), (0, 1)])
    for k in range(nz):
        kk = np.full_like(ii, k)
        if k < n_hex:
            hexes.append(np.stack([nid(ii + a, jj + b, kk + c) for a, b, c in corners], axis=1))
        elif k < n_hex + n_wedge:
            layer = []
            for tri in tris:
                bot = [nid(ii + a, jj + b, kk) for a, b in tri]
                top = [nid(ii + a, jj + b, kk + 1) for a, b in tri]
                layer.append(np.stack(bot + top, axis=1))
            prisms.append(np.stack(layer, axis=1).reshape(-1, 6))
        else:
            cell = []
            for perm in itertools.permutations(range(3)):
                off = [0, 0, 0]
                verts = [nid(ii, jj, kk)]
                for ax in perm:
                    off[ax] += 1
                    verts.append(nid(ii + off[0], jj + off[1], kk + off[2]))
                cell.append(np.stack(verts, axis=1))
            tets.append(np.stack(cell, axis=1).reshape(-1, 4))
    cat = lambda lst, w: np.concatenate(lst).astype(np.int32) if lst else np.zeros((0, w), np.int32)  # noqa: E731
    ien = _orient(cat(tets, 4), x).astype(np.int32) if tets else np.zeros((0, 4), np.int32)
    h = min(lengths[0] / nxy, lengths[1] / nxy, lengths[2] / nz)
    BC = np.zeros((6, x.shape[0]))
    bnd, ienb = [], np.zeros((0, 4), np.int32)
    if not periodic_x:
        _inflow(x, iBC, BC, inflow)
        ienb = _tet_x_faces(x, ien, lengths[0])
        jj1 = np.arange(nxy)
        for lcsyst, k0, k1, fn in ((2, 0, n_hex, _hex_x_faces), (4, n_hex, n_hex + n_wedge, _wedge_x_faces)):
            if k1 > k0:
                j2, k2 = (a.reshape(-1) for a in np.meshgrid(jj1, np.arange(k0, k1), indexing="ij"))
                bnd.append(bnd_block(lcsyst, fn(nid, nxy, j2, k2)))
    nb = ienb.shape[0]
    return Case(nshg=x.shape[0], x=x, ien=ien, ienb=ienb, iBCB=np.zeros((nb, 2), np.int32),
                BCB=np.zeros((nb, 3, 6)), iBC=iBC, BC=BC, iper=iper, h=h,
                ienh=cat(hexes, 8), ienw=cat(prisms, 6), bnd=bnd,
                meta={"n": n, "lengths": lengths, "periodic": (periodic_x, True, True),
                      "layers": (n_hex, n_wedge, n_tet)})


def concat(*cases: Case) -> Case:
    """Disjoint union of meshes (node numbers of each part offset by the nodes before it)."""
    off = 0
    parts = {k: [] for k in ("x", "ien", "ienb", "iBCB", "BCB", "iBC", "BC", "iper", "ienh", "ienw")}
    for c in cases:
        parts["x"].append(c.x)
        parts["ien"].append(c.ien + off)
        parts["ienb"].append(c.ienb + off)
        parts["iBCB"].append(c.iBCB)
        parts["BCB"].append(c.BCB)
        parts["iBC"].append(c.iBC)
        parts["BC"].append(c.BC)
        parts["iper"].append(c.iper + off)
        parts["ienh"].append(c.ienh + off)
        parts["ienw"].append(c.ienw + off)
        off += c.nshg
    cat = {k: np.concatenate(v, axis=(1 if k == "BC" else 0)) for k, v in parts.items()}
    bnd, boff = {}, 0
    for c in cases:
        for b in c.bnd:
            bnd.setdefault(b.lcsyst, []).append(BndBlock(b.lcsyst, b.ien + boff, b.iBCB, b.BCB))
        boff += c.nshg
    bnd = [BndBlock(l, np.concatenate([b.ien for b in v]).astype(np.int32), np.concatenate([b.iBCB for b in v]),
                    np.concatenate([b.BCB for b in v])) for l, v in sorted(bnd.items())]
    return Case(nshg=off, x=cat["x"], ien=cat["ien"].astype(np.int32), ienb=cat["ienb"].astype(np.int32),
                iBCB=cat["iBCB"].astype(np.int32), BCB=cat["BCB"], iBC=cat["iBC"].astype(np.int32), BC=cat["BC"],
                iper=cat["iper"].astype(np.int32), h=min(c.h for c in cases), ienh=cat["ienh"].astype(np.int32),
                ienw=cat["ienw"].astype(np.int32), meta={"parts": [c.meta for c in cases]}, bnd=bnd)


def renumber(case: Case, new_of_old: np.ndarray) -> Case:
    """The same mesh with node n renamed new_of_old[n] (elements, faces and their order unchanged)."""
    p = np.asarray(new_of_old, dtype=np.int64)
    N = case.nshg
    if p.shape != (N,) or not np.array_equal(np.sort(p), np.arange(N)):
        raise ValueError("new_of_old must be a permutation of the nodes")
    old_of_new = np.empty(N, np.int64)
    old_of_new[p] = np.arange(N)
    return Case(nshg=N, x=np.ascontiguousarray(case.x[old_of_new]), ien=p[case.ien].astype(np.int32),
                ienb=p[case.ienb].astype(np.int32), iBCB=case.iBCB.copy(), BCB=case.BCB.copy(),
                iBC=case.iBC[old_of_new].astype(np.int32), BC=np.ascontiguousarray(case.BC[:, old_of_new]),
                iper=p[case.iper[old_of_new]].astype(np.int32), h=case.h, meta=dict(case.meta),
                ienh=p[case.ienh].astype(np.int32), ienw=p[case.ienw].astype(np.int32),
                bnd=[BndBlock(b.lcsyst, p[b.ien].astype(np.int32), b.iBCB.copy(), b.BCB.copy()) for b in case.bnd])


def renumber_field(v: np.ndarray, new_of_old: np.ndarray, ncomp: int) -> np.ndarray:
    """A nodal field in the reference's column-major (nshg, ncomp) layout, renumbered."""
    p = np.asarray(new_of_old, dtype=np.int64)
    old_of_new = np.empty_like(p)
    old_of_new[p] = np.arange(p.size)
    return np.ascontiguousarray(np.asarray(v).reshape(ncomp, -1)[:, old_of_new]).reshape(-1)


# ---------------------------------------------------------------------------
# seeded states (counter-based: the value of (node, dof) does not depend on
# the mesh size or traversal order)
# ---------------------------------------------------------------------------
def _noise(seed: int, nshg: int, ndof: int = 5) -> np.ndarray:
    """Standard normals from a Philox counter generator keyed by seed; row k = dof k."""
    g = np.random.Generator(np.random.Philox(key=seed))
    return g.standard_normal((ndof, nshg))


def freestream(mach: float, u: float = 1.0, rho: float = 1.0) -> dict:
    R = rgas()
    c = u / mach
    T = c * c / (GAMMA * R)
    p = rho * R * T
    return {"u": u, "T": T, "p": p, "c": c, "rho": rho}


def uniform_state(case: Case, mach: float, sigma: float = 0.01, seed: int = 20261203) -> np.ndarray:
    """y(nshg,5) in the reference order (u,v,w,p,T), column-major flat (5*nshg)."""
    fs = freestream(mach)
    y = np.empty((5, case.nshg))
    y[0], y[1], y[2], y[3], y[4] = fs["u"], 0.0, 0.0, fs["p"], fs["T"]
    if sigma > 0:
        z = _noise(seed, case.nshg)
        scale = np.array([fs["u"], fs["u"], fs["u"], fs["p"], fs["T"]])[:, None]
        y += sigma * scale * z
    return apply_bc_state(case, y.reshape(-1))


def vortex_state(case: Case, mach: float = 0.1, noise: float = 1e-3, seed: int = 20261203) -> np.ndarray:
    """u = U0 sin x cos y cos z, v = -U0 cos x sin y cos z, w = 0, uniform p and T, + noise."""
    fs = freestream(mach)
    X, Yc, Z = case.x[:, 0], case.x[:, 1], case.x[:, 2]
    y = np.empty((5, case.nshg))
    y[0] = np.sin(X) * np.cos(Yc) * np.cos(Z)
    y[1] = -np.cos(X) * np.sin(Yc) * np.cos(Z)
    y[2] = 0.0
    y[3], y[4] = fs["p"], fs["T"]
    if noise > 0:
        z = _noise(seed, case.nshg)
        scale = np.array([1.0, 1.0, 1.0, fs["p"], fs["T"]])[:, None]
        y += noise * scale * z
    return apply_bc_state(case, y.reshape(-1))


def fourier_state(case: Case, mach: float, kmax: int = 8, nmodes: int = 24, noise: float = 0.0,
                  seed: int = 20261203, lengths=None) -> np.ndarray:
    """Random-phase Fourier velocity modes: u(x) = sum_m a_m cos(2 pi k_m . x / L + phi_m) with
    integer wave vectors 1 <= |k_m|_inf <= kmax and amplitudes a_m perpendicular to k_m
    (divergence-free), scaled so that max |u| over the nodes is 1; p and T of the free stream at
    ``mach`` (so max |u| / c = mach), plus ``noise`` x seeded Gaussian noise."""
    fs = freestream(mach)
    g = np.random.default_rng(seed)
    L = np.asarray(lengths if lengths is not None else case.meta.get("lengths", (1.0, 1.0, 1.0)), dtype=np.float64)
    x = case.x
    u = np.zeros((case.nshg, 3))
    for _ in range(nmodes):
        k = np.zeros(3)
        while not np.any(k):
            k = g.integers(-kmax, kmax + 1, size=3).astype(np.float64)
        a = g.standard_normal(3)
        a -= k * (a @ k) / (k @ k)
        a /= np.linalg.norm(a) * np.sqrt(k @ k)  # energy falling with |k|
        phi = g.uniform(0.0, 2.0 * np.pi)
        u += np.cos(2.0 * np.pi * (x / L) @ k + phi)[:, None] * a[None, :]
    u /= np.abs(np.linalg.norm(u, axis=1)).max()
    y = np.empty((5, case.nshg))
    y[0], y[1], y[2] = u[:, 0], u[:, 1], u[:, 2]
    y[3], y[4] = fs["p"], fs["T"]
    if noise > 0:
        z = _noise(seed + 1, case.nshg)
        y += noise * np.array([1.0, 1.0, 1.0, fs["p"], fs["T"]])[:, None] * z
    return apply_bc_state(case, y.reshape(-1))


def apply_bc_state(case: Case, y: np.ndarray) -> np.ndarray:
    """itrBC for Dirichlet T/velocity and the periodic master->slave copy (itrbc.f:54-176)."""
    y = y.reshape(5, case.nshg).copy()
    ib = case.iBC
    t = (ib >> 1) & 1 == 1
    y[4, t] = case.BC[1, t]
    v7 = ((ib >> 3) & 7) == 7
    y[0, v7], y[1, v7], y[2, v7] = case.BC[2, v7], case.BC[3, v7], case.BC[4, v7]
    y = y[:, case.iper]
    return np.ascontiguousarray(y).reshape(-1)


def time_params(rho_inf: float, dt: float) -> dict:
    """Generalized-alpha parameters of itrSetup (itrPC.f:16-24, 42)."""
    if rho_inf < 0 or rho_inf > 1:
        almi = alfi = gami = 1.0
    else:
        almi = (3.0 - rho_inf) / (1.0 + rho_inf) / 2.0
        alfi = 1.0 / (1.0 + rho_inf)
        gami = 0.5 + almi - alfi
    return {"Dtgl": 1.0 / dt, "almi": almi, "alfi": alfi, "gami": gami}


def cfl_dt(case: Case, mach: float, cfl: float = 1.0, umax: float = 1.0) -> float:
    fs = freestream(mach, u=umax)
    return cfl * case.h / (umax + fs["c"])


# ---------------------------------------------------------------------------
# benchmark cases (sizes of the reference's benchmark definitions)
# ---------------------------------------------------------------------------
def channel_case(n: int, mach: float = 0.3, re: float = 1000.0):
    """Unit cube, periodic y/z, Dirichlet inflow at x=0, natural outflow at x=1."""
    fs = freestream(mach)
    case = box(n, periodic=(False, True, True), inflow={"T": fs["T"], "u": (fs["u"], 0.0, 0.0)})
    mu = fs["rho"] * fs["u"] * 1.0 / re
    dt = cfl_dt(case, mach)
    return case, {"mach": mach, "re": re, "mu": mu, "dt": dt, "fs": fs}


def channel_hex_case(n, mach: float = 0.3, re: float = 1000.0):
    """The channel on n^3 hexes: periodic y/z, Dirichlet inflow at x = 0, natural outflow at
    x = 1 through boundary hexes (lcsyst 2)."""
    fs = freestream(mach)
    case = hex_box(n, periodic=(False, True, True), inflow={"T": fs["T"], "u": (fs["u"], 0.0, 0.0)})
    mu = fs["rho"] * fs["u"] * 1.0 / re
    return case, {"mach": mach, "re": re, "mu": mu, "dt": cfl_dt(case, mach), "fs": fs}


def channel_wedge_case(n, mach: float = 0.3, re: float = 1000.0):
    """The channel on prisms: periodic y, Dirichlet inflow at x = 0 and natural outflow at x = 1
    through quadrilateral faces (lcsyst 4), natural walls at z = 0 and z = 1 through triangle
    faces (lcsyst 3)."""
    fs = freestream(mach)
    case = wedge_box(n, periodic=(False, True, False), inflow={"T": fs["T"], "u": (fs["u"], 0.0, 0.0)})
    mu = fs["rho"] * fs["u"] * 1.0 / re
    return case, {"mach": mach, "re": re, "mu": mu, "dt": cfl_dt(case, mach), "fs": fs}


def periodic_vortex_case(n: int, mach: float = 0.1, re: float = 1600.0):
    L = 2.0 * math.pi
    case = box(n, lengths=(L, L, L), periodic=(True, True, True), inflow=None)
    fs = freestream(mach)
    mu = fs["rho"] * 1.0 * 1.0 / re
    dt = cfl_dt(case, mach)
    return case, {"mach": mach, "re": re, "mu": mu, "dt": dt, "fs": fs}


def layered_case(nxy: int, n_hex: int, n_wedge: int, n_tet: int, mach: float = 0.3, re: float = 1000.0,
                 periodic_x: bool = True):
    """The connected mixed-topology box of ``layered`` with the channel's physics; with
    ``periodic_x`` False a Dirichlet inflow at x = 0 and natural outflow at x = 1 through
    boundary tets, hexes and prisms."""
    fs = freestream(mach)
    case = layered(nxy, n_hex, n_wedge, n_tet, periodic_x=periodic_x,
                   inflow=None if periodic_x else {"T": fs["T"], "u": (fs["u"], 0.0, 0.0)})
    mu = fs["rho"] * fs["u"] * 1.0 / re
    dt = cfl_dt(case, mach)
    return case, {"mach": mach, "re": re, "mu": mu, "dt": dt, "fs": fs}


def mixed_case(n_tet=4, n_hex=4, n_wedge=(4, 4, 2), mach: float = 0.3, re: float = 1000.0):
    """Three disjoint periodic unit boxes: n_tet^3 x 6 tets, n_hex^3 hexes and 2 x prod(n_wedge)
    wedges -- the element blocks of a mixed-topology mesh (each block conforming)."""
    parts = []
    if n_tet:
        parts.append(box(n_tet, periodic=(True, True, True), inflow=None))
    if n_hex:
        parts.append(hex_box(n_hex))
    if n_wedge:
        parts.append(wedge_box(n_wedge))
    case = concat(*parts)
    fs = freestream(mach)
    mu = fs["rho"] * fs["u"] * 1.0 / re
    dt = cfl_dt(case, mach)
    return case, {"mach": mach, "re": re, "mu": mu, "dt": dt, "fs": fs}
