"""ctypes wrapper of the oracle (libphoracle.so) -- test infrastructure only.

The same method names and array layouts as phasta_gb300.solver.GpuSolver, so
parity tests compare the two call for call.  Only tests/, the smoke check and
the CPU-baseline leg of bench.py use this module.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Common(C.Structure):
    _fields_ = [
        ("Rgas", C.c_double), ("gamma", C.c_double), ("gamma1", C.c_double), ("pr", C.c_double),
        ("rmu", C.c_double), ("Dtgl", C.c_double), ("almi", C.c_double), ("alfi", C.c_double),
        ("gami", C.c_double), ("dtsfct", C.c_double), ("taucfct", C.c_double), ("temper", C.c_double),
        ("itau", C.c_int), ("ivart", C.c_int), ("iremoveStabTimeTerm", C.c_int), ("Navier", C.c_int),
        ("ipord", C.c_int), ("EntropyPressure", C.c_int), ("Kspace", C.c_int), ("nGMRES", C.c_int),
        ("minIters", C.c_int), ("etol", C.c_double), ("epsM", C.c_double), ("eGMRES", C.c_double),
        ("iter", C.c_int), ("istep", C.c_int), ("idiff", C.c_int), ("iDC", C.c_int),
    ]


class OBnd(C.Structure):
    _fields_ = [("lcsyst", C.c_int), ("nelem", C.c_int), ("ien", _ip), ("iBCB", _ip), ("BCB", _dp)]


class OMesh(C.Structure):
    _fields_ = [
        ("nshg", C.c_int), ("nelem", C.c_int), ("ien", _ip), ("nblk", C.c_int), ("blk_start", _ip),
        ("ngrp", C.c_int), ("grp_start", _ip), ("x", _dp), ("nbelem", C.c_int), ("ienb", _ip),
        ("iBCB", _ip), ("BCB", _dp), ("iBC", _ip), ("BC", _dp), ("iper", _ip),
        ("nhex", C.c_int), ("ienh", _ip), ("nwedge", C.c_int), ("ienw", _ip),
        ("nbblk", C.c_int), ("bblk", C.POINTER(OBnd)),
    ]


class OStats(C.Structure):
    _fields_ = [("iKs", C.c_int), ("lGMRES", C.c_int), ("ntotGM", C.c_int), ("unorm0", C.c_double),
                ("echeck", C.c_double), ("eGMRES", C.c_double), ("totres", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        from .build_oracle import build_oracle  # noqa: WPS433
        build_oracle()
        L = C.CDLL(str(HERE / "libphoracle.so"))
        cp, mp, vp = C.POINTER(Common), C.POINTER(OMesh), None
        sig = {
            "or_make_groups": ([C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, _ip, _ip, C.c_int], C.c_int),
            "or_tet_tables": ([_dp] * 6, None),
            "or_topo_tables": ([C.c_int, _dp, _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int)], None),
            "or_btopo_tables": ([C.c_int, _dp, _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int), _ip], None),
            "or_e3": ([cp, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp], None),
            "or_e3b": ([cp, C.c_int, _dp, _ip, _dp, _dp, _dp], None),
            "or_elmmfg": ([cp, mp, _dp, _dp, _dp, _dp, _dp, C.c_int, C.c_int], None),
            "or_itrres": ([cp, mp, _dp, _dp, _dp, _dp, C.c_int, C.c_int], None),
            "or_elmres": ([cp, mp, _dp, _dp, _dp, C.c_int], None),
            "or_bc3res": ([mp, _dp, _dp, cp], None),
            "or_bc3bdg": ([mp, _dp, _dp, cp], None),
            "or_itrbc": ([mp, _dp, _dp, C.c_int, C.c_double], None),
            "or_i3lu": ([C.c_int, _dp, _dp, C.c_int], None),
            "or_yshuffle": ([C.c_int, _dp, C.c_int], None),
            "or_solmfg": ([cp, mp, _dp, _dp, _dp, _dp, _dp, C.POINTER(OStats), C.c_int], None),
            "or_genadj": ([mp, C.c_int, _ip, _ip, C.POINTER(C.c_int)], C.c_int),
            "or_elmgmrs": ([cp, mp, _dp, _dp, _ip, _ip, C.c_int, _dp, _dp, _dp, C.c_int], None),
            "or_spsi3pre": ([C.c_int, _ip, _ip, _dp, _dp], None),
            "or_sparseap": ([mp, _ip, _ip, _dp, _dp], None),
            "or_solgmrs": ([cp, mp, _ip, _ip, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(OStats), C.c_int],
                           None),
            "or_elmgmre": ([cp, mp, _ip, _dp, _dp, _dp, _dp, _dp, C.c_int], None),
            "or_i3pre": ([mp, _ip, _dp, _dp], None),
            "or_au1gmr": ([mp, _ip, _dp, _dp], None),
            "or_solgmre": ([cp, mp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(OStats), C.c_int], None),
            "or_itrpredict": ([cp, C.c_int, _dp, _dp, _dp, _dp], None),
            "or_itrcorrect": ([cp, C.c_int, _dp, _dp, _dp, _dp, _dp], None),
            "or_itrupdate": ([cp, C.c_int, _dp, _dp, _dp, _dp], None),
        }
        for name, (a, r) in sig.items():
            f = getattr(L, name)
            f.argtypes = a
            f.restype = r
        _lib = L
    return _lib


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _i(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def common(params: dict) -> Common:
    c = Common()
    for name, _ in Common._fields_:
        if name in params:
            setattr(c, name, params[name])
    return c


@dataclass
class OracleStats:
    iKs: int
    lGMRES: int
    ntotGM: int
    unorm0: float
    echeck: float
    eGMRES: float
    totres: float


def tet_tables():
    L = lib()
    shp, shgl, qwt = np.zeros(16), np.zeros(48), np.zeros(4)
    shpb, shglb, qwtb = np.zeros(12), np.zeros(36), np.zeros(3)
    L.or_tet_tables(_d(shp), _d(shgl), _d(qwt), _d(shpb), _d(shglb), _d(qwtb))
    return {"shp": shp.reshape(4, 4), "shgl": shgl.reshape(4, 3, 4), "Qwt": qwt,
            "shpb": shpb.reshape(3, 4), "shglb": shglb.reshape(3, 3, 4), "Qwtb": qwtb}


def e3(params: dict, yl, ycl, acl, xl, ires=3, iprec=1):
    """One element (e3.f). yl/ycl/acl (4,5) in element order (p,u,v,w,T), xl (4,3)."""
    L = lib()
    c = common(params)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    rl, rml, bd = np.zeros((4, 5)), np.zeros((4, 5)), np.zeros((4, 5, 5))
    L.or_e3(C.byref(c), ires, iprec, _d(f(yl)), _d(f(ycl)), _d(f(acl)), _d(f(xl)), _d(rl), _d(rml), _d(bd))
    return rl, rml, bd


class Oracle:
    """The whole-mesh routines on a Case (phasta_gb300.mesh.Case)."""

    def __init__(self, case, params: dict, nthreads: int = 1, grouped: bool | None = None, bksiz: int = 64):
        self.L = lib()
        self.case = case
        self.params = dict(params)
        self.nthreads = nthreads
        self.nshg = case.nshg
        grouped = nthreads > 1 if grouped is None else grouped
        grouped = grouped and case.nelem > 0  # the groups order the tet block
        ien = np.ascontiguousarray(case.ien, dtype=np.int32)
        E = ien.shape[0]
        if grouped:
            perm = np.zeros(E, np.int32)
            blk = np.zeros(E + 2, np.int32)
            grp = np.zeros(1025, np.int32)
            nb = C.c_int()
            ng = self.L.or_make_groups(self.nshg, E, _i(ien.reshape(-1)), bksiz, _i(perm), _i(blk), C.byref(nb),
                                       _i(grp), 1024)
            assert ng > 0
            ien = np.ascontiguousarray(ien[perm])
            self._eid = np.ascontiguousarray(perm, dtype=np.int32)
            self._blk = np.ascontiguousarray(blk[: nb.value + 1])
            self._grp = np.ascontiguousarray(grp[: ng + 1])
            ngrp = ng
        else:
            nb = (E + bksiz - 1) // bksiz
            self._blk = np.minimum(np.arange(nb + 1, dtype=np.int32) * bksiz, E).astype(np.int32)
            self._grp = np.zeros(1, np.int32)
            ngrp = 0
            self._eid = np.arange(E, dtype=np.int32)
        self._ien = ien.reshape(-1)
        self._x = case.x_ref()
        self._ienb = np.ascontiguousarray(case.ienb, dtype=np.int32).reshape(-1)
        self._iBCB = np.ascontiguousarray(case.iBCB, dtype=np.int32).reshape(-1)
        self._BCB = np.ascontiguousarray(case.BCB, dtype=np.float64).reshape(-1)
        self._iBC = np.ascontiguousarray(case.iBC, dtype=np.int32)
        self._BC = np.ascontiguousarray(case.BC, dtype=np.float64).reshape(-1)
        self._iper = np.ascontiguousarray(case.iper, dtype=np.int32)
        self._ienh = np.ascontiguousarray(getattr(case, "ienh", np.zeros((0, 8))), dtype=np.int32).reshape(-1)
        self._ienw = np.ascontiguousarray(getattr(case, "ienw", np.zeros((0, 6))), dtype=np.int32).reshape(-1)
        bnd = getattr(case, "bnd", [])
        self._bnd_arrays = [(np.ascontiguousarray(b.ien, dtype=np.int32).reshape(-1),
                             np.ascontiguousarray(b.iBCB, dtype=np.int32).reshape(-1),
                             np.ascontiguousarray(b.BCB, dtype=np.float64).reshape(-1)) for b in bnd]
        self._bblk = (OBnd * max(1, len(bnd)))(*[OBnd(b.lcsyst, b.ien.shape[0], _i(a[0]), _i(a[1]), _d(a[2]))
                                                 for b, a in zip(bnd, self._bnd_arrays)])
        self.m = OMesh(self.nshg, E, _i(self._ien), len(self._blk) - 1, _i(self._blk), ngrp, _i(self._grp),
                       _d(self._x), case.nbelem, _i(self._ienb), _i(self._iBCB), _d(self._BCB), _i(self._iBC),
                       _d(self._BC), _i(self._iper), len(self._ienh) // 8, _i(self._ienh), len(self._ienw) // 6,
                       _i(self._ienw), len(bnd), self._bblk)
        self.c = common(self.params)
        self.ntotGM = 0

    def set_params(self, **kw):
        self.params.update(kw)
        self.c = common(self.params)

    def _v(self, k=5):
        return np.zeros(k * self.nshg)

    def ElmMFG(self, y, ac, iprec=1):
        res, rmes, bd = self._v(), self._v(), self._v(25)
        self.L.or_elmmfg(C.byref(self.c), C.byref(self.m), _d(y), _d(ac), _d(res), _d(rmes), _d(bd), iprec,
                         self.nthreads)
        return res, rmes, (bd if iprec else None)

    def ElmRes(self, y, ac):
        res = self._v()
        self.L.or_elmres(C.byref(self.c), C.byref(self.m), _d(y), _d(ac), _d(res), self.nthreads)
        return res

    def ItrRes(self, yp, yc, ac, rmes=None, iabres=0):
        rmes = self._v() if rmes is None else np.array(rmes, dtype=np.float64)
        self.L.or_itrres(C.byref(self.c), C.byref(self.m), _d(yp), _d(yc), _d(ac), _d(rmes), iabres, self.nthreads)
        return rmes

    def i3LU(self, bd, r, code):
        bd = np.array(bd, dtype=np.float64)
        r = None if r is None else np.array(r, dtype=np.float64)
        self.L.or_i3lu(self.nshg, _d(bd), _d(r), code)
        return bd, r

    def bc3Res(self, y, res):
        res = np.array(res, dtype=np.float64)
        self.L.or_bc3res(C.byref(self.m), _d(y), _d(res), C.byref(self.c))
        return res

    def bc3BDg(self, y, bd):
        bd = np.array(bd, dtype=np.float64)
        self.L.or_bc3bdg(C.byref(self.m), _d(y), _d(bd), C.byref(self.c))
        return bd

    def itrBC(self, y, ac=None, ires=3):
        y = np.array(y, dtype=np.float64)
        ac = None if ac is None else np.array(ac, dtype=np.float64)
        self.L.or_itrbc(C.byref(self.m), _d(y), _d(ac), ires, self.params["Rgas"])
        return y, ac

    def SolMFG(self, y, ac):
        res, bd, Dy = self._v(), self._v(25), self._v()
        st = OStats()
        st.ntotGM = self.ntotGM
        self.L.or_solmfg(C.byref(self.c), C.byref(self.m), _d(y), _d(ac), _d(res), _d(bd), _d(Dy), C.byref(st),
                         self.nthreads)
        self.ntotGM = st.ntotGM
        self.params["eGMRES"] = self.c.eGMRES
        return res, bd, Dy, OracleStats(st.iKs, st.lGMRES, st.ntotGM, st.unorm0, st.echeck, st.eGMRES, st.totres)

    # ---- sparse solver (lhs = 1): colm/rowp 1-based, lhsK (nnz_tot, 25) = the reference's lhsK(25, nnz_tot)
    def genadj(self, nnz: int = 40):
        colm = np.zeros(self.nshg + 1, np.int32)
        rowp = np.zeros(self.nshg * nnz, np.int32)
        icnt = C.c_int()
        if self.L.or_genadj(C.byref(self.m), nnz, _i(colm), _i(rowp), C.byref(icnt)) != 0:
            raise ValueError("genadj: more than nnz blocks in a row")
        self.colm, self.rowp = colm, np.ascontiguousarray(rowp[: icnt.value])
        return self.colm.copy(), self.rowp.copy()

    def _adj(self):
        if not hasattr(self, "colm"):
            self.genadj()
        return self.colm, self.rowp

    def ElmGMRs(self, y, ac):
        colm, rowp = self._adj()
        res, bd = self._v(), self._v(25)
        lhsK = np.zeros((len(rowp), 25))
        self.L.or_elmgmrs(C.byref(self.c), C.byref(self.m), _d(y), _d(ac), _i(colm), _i(rowp), len(rowp), _d(res),
                          _d(bd), _d(lhsK), self.nthreads)
        return res, bd, lhsK

    def Spsi3pre(self, lu, lhsK):
        colm, rowp = self._adj()
        out = np.array(lhsK, dtype=np.float64, order="C")
        self.L.or_spsi3pre(self.nshg, _i(colm), _i(rowp), _d(np.ascontiguousarray(lu, dtype=np.float64)), _d(out))
        return out

    def SparseAp(self, lhsK, p):
        colm, rowp = self._adj()
        p = np.array(p, dtype=np.float64)
        self.L.or_sparseap(C.byref(self.m), _i(colm), _i(rowp), _d(np.ascontiguousarray(lhsK, dtype=np.float64)),
                           _d(p))
        return p

    def SolGMRs(self, y, ac, lGMRES_common: int = 0):
        colm, rowp = self._adj()
        res, bd, Dy = self._v(), self._v(25), self._v()
        lhsK = np.zeros((len(rowp), 25))
        st = OStats()
        st.ntotGM = self.ntotGM
        st.lGMRES = lGMRES_common
        self.L.or_solgmrs(C.byref(self.c), C.byref(self.m), _i(colm), _i(rowp), len(rowp), _d(y), _d(ac), _d(res),
                          _d(bd), _d(Dy), _d(lhsK), C.byref(st), self.nthreads)
        self.ntotGM = st.ntotGM
        return res, bd, Dy, lhsK, OracleStats(st.iKs, st.lGMRES, st.ntotGM, st.unorm0, st.echeck, st.eGMRES,
                                              st.totres)

    # ---- element-by-element solver: EG (numel, nedof, nedof) = the reference's EGmass
    def _eg(self):
        n = self.case.nelem + self.case.nhex + self.case.nwedge
        nd = 40 if self.case.nhex else 30 if self.case.nwedge else 20
        return np.zeros((nd, nd, n))  # C order (j, i, e) = Fortran (e, i, j)

    def ElmGMRe(self, y, ac):
        res, bd, EG = self._v(), self._v(25), self._eg()
        self.L.or_elmgmre(C.byref(self.c), C.byref(self.m), _i(self._eid), _d(y), _d(ac), _d(res), _d(bd), _d(EG),
                          self.nthreads)
        return res, bd, EG.transpose(2, 1, 0)

    def i3pre(self, lu, EG):
        out = np.ascontiguousarray(np.asarray(EG).transpose(2, 1, 0))
        self.L.or_i3pre(C.byref(self.m), _i(self._eid), _d(np.ascontiguousarray(lu, dtype=np.float64)), _d(out))
        return out.transpose(2, 1, 0)

    def Au1GMR(self, EG, p):
        p = np.array(p, dtype=np.float64)
        eg = np.ascontiguousarray(np.asarray(EG).transpose(2, 1, 0))
        self.L.or_au1gmr(C.byref(self.m), _i(self._eid), _d(eg), _d(p))
        return p

    def SolGMRe(self, y, ac):
        res, bd, Dy, EG = self._v(), self._v(25), self._v(), self._eg()
        st = OStats()
        st.ntotGM = self.ntotGM
        self.L.or_solgmre(C.byref(self.c), C.byref(self.m), _i(self._eid), _d(y), _d(ac), _d(res), _d(bd), _d(Dy),
                          _d(EG), C.byref(st), self.nthreads)
        self.ntotGM = st.ntotGM
        return res, bd, Dy, EG.transpose(2, 1, 0), OracleStats(st.iKs, st.lGMRES, st.ntotGM, st.unorm0, st.echeck,
                                                               st.eGMRES, st.totres)

    def itrPredict(self, yold, acold):
        y, ac = self._v(), self._v()
        self.L.or_itrpredict(C.byref(self.c), self.nshg, _d(yold), _d(acold), _d(y), _d(ac))
        return y, ac

    def itrCorrect(self, y, ac, yold, acold, Dy):
        y, ac = np.array(y, dtype=np.float64), np.array(ac, dtype=np.float64)
        self.L.or_itrcorrect(C.byref(self.c), self.nshg, _d(y), _d(ac), _d(yold), _d(acold), _d(Dy))
        y, ac = self.itrBC(y, ac, ires=3)
        return y, ac

    def itrUpdate(self, yold, acold, y, ac):
        yold, acold = np.array(yold, dtype=np.float64), np.array(acold, dtype=np.float64)
        self.L.or_itrupdate(C.byref(self.c), self.nshg, _d(yold), _d(acold), _d(y), _d(ac))
        return self.itrBC(yold, acold, ires=3)

    def newton(self, y, ac, yold, acold):
        """SolMFG + itrCorrect + itrBC (itrdrv.f:489-598)."""
        res, bd, Dy, st = self.SolMFG(y, ac)
        y, ac = self.itrCorrect(y, ac, yold, acold, Dy)
        return y, ac, st, Dy

    def time_step(self, yold, acold, nitr):
        y, ac = self.itrPredict(yold, acold)
        y, ac = self.itrBC(y, ac, ires=3)
        stats = []
        for it in range(1, nitr + 1):
            self.set_params(iter=it)
            y, ac, st, _ = self.newton(y, ac, yold, acold)
            stats.append(st)
        yold, acold = self.itrUpdate(yold, acold, y, ac)
        self.set_params(istep=self.params["istep"] + 1)
        return yold, acold, y, ac, stats


def btopo_tables(lcsyst: int) -> dict:
    """Boundary quadrature/shape tables of boundary topology lcsyst (2 hex, 3 wedge triangle face,
    4 wedge quadrilateral face): shpb[q][a], shglb[q][i][a], Qwtb[q], lnode (0-based face nodes)."""
    L = lib()
    shp, shgl, qwt = np.zeros(32), np.zeros(96), np.zeros(4)
    nshl, nshlb, ng = C.c_int(), C.c_int(), C.c_int()
    ln = np.zeros(4, np.int32)
    L.or_btopo_tables(lcsyst, _d(shp), _d(shgl), _d(qwt), C.byref(nshl), C.byref(nshlb), C.byref(ng), _i(ln))
    n, q = nshl.value, ng.value
    return {"shpb": shp[: q * n].reshape(q, n), "shglb": shgl[: 3 * q * n].reshape(q, 3, n), "Qwtb": qwt[:q],
            "lnode": ln[: nshlb.value].copy()}


def topo_tables(lcsyst: int) -> dict:
    """Quadrature/shape tables of topology lcsyst (1 tet, 2 hex, 3 wedge): shp[q][a], shgl[q][i][a], Qwt[q]."""
    L = lib()
    shp, shgl, qwt = np.zeros(64), np.zeros(192), np.zeros(8)
    nshl, ng = C.c_int(), C.c_int()
    L.or_topo_tables(lcsyst, _d(shp), _d(shgl), _d(qwt), C.byref(nshl), C.byref(ng))
    n, q = nshl.value, ng.value
    return {"shp": shp[: q * n].reshape(q, n), "shgl": shgl[: 3 * q * n].reshape(q, 3, n), "Qwt": qwt[:q]}
