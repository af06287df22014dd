"""The reference's own Fortran routines of the hot path, run through fexec.

``RefPhasta(case, params, root)`` loads the reference sources below from the
reference tree ``root`` (its ``phSolver`` directory), sets the COMMON blocks a
single-rank PHASTA run would hold for one linear-tet interior block and one
boundary block, and exposes the routines with host arrays in the layouts of
``include/phgpu.h`` (``y[k*nshg + n]``, ``bd[(i + 5j)*nshg + n]``).  It only
runs where the reference tree is present; ``make_ref_golden.py`` uses it to
write the committed golden vectors.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

try:
    from . import fexec
except ImportError:  # run as a script from tests/golden
    import fexec

HERE = Path(__file__).resolve().parent

SOURCES = [
    # ElmMFG chain
    "compressible/elmmfg.f", "compressible/asimfg.f", "common/local.f", "common/localy.f",
    "compressible/e3.f", "common/hierarchic.f", "compressible/e3ivar.f", "compressible/getthm.f",
    "compressible/getdiff.f", "common/e3metric.f", "compressible/e3mtrx.f", "compressible/e3conv.f",
    "compressible/e3visc.f", "compressible/e3ls.f", "compressible/e3tau.f", "compressible/e3massr.f",
    "compressible/e3bdg.f", "compressible/e3wmlt.f",
    # boundary elements and boundary conditions
    "compressible/asbmfg.f", "compressible/e3b.f", "compressible/e3bvar.f", "compressible/bc3res.f",
    "compressible/bc3bdg.f", "compressible/bc3per.f", "compressible/itrbc.f",
    # solver
    "compressible/itrres.f", "compressible/asires.f", "compressible/i3lu.f", "compressible/solmfg.f",
    "compressible/au1mfg.f", "compressible/au2mfg.f", "compressible/itrfdi.f", "compressible/shuffle.f",
    "compressible/itrPC.f", "common/mpitools.f", "common/clear.f",
    # idiff = 1: global reconstruction of the diffusive flux
    "compressible/asiq.f", "compressible/e3q.f", "compressible/e3qvar.f", "common/qpbc.f",
    # assembled tangent: ElmGMRs, AsIGMR, e3massl, bc3LHS, fillsparseC, genadj/Asadj,
    # Spsi3pre, SparseAp, SolGMRs
    "compressible/elmgmr.f", "compressible/asigmr.f", "compressible/e3massl.f", "compressible/bc3lhs.f",
    "common/fillsparse.f", "common/genadj.f", "common/asadj.f", "compressible/spsi3pre.f",
    "compressible/sparseap.f", "compressible/solgmr.f",
    # element-by-element solver: ElmGMRe, i3pre, Au1GMR/AsAuGMR/localt, SolGMRe
    "compressible/i3pre.f", "compressible/au1gmr.f", "compressible/asaugmr.f", "compressible/localt.f",
    # discontinuity capturing (iDC = 1, 2, 3)
    "compressible/e3dc.f",
]
# rstat.f only prints statistics, and SolMFG calls it with two of its three
# arguments (solmfg.f:367 vs rstat.f:1); its totres (rstat.f:108) is computed
# from the returned residual instead.

MODULES = ["rlssave", "turbsa", "specialbc", "turbke", "spat_var_eps", "timedata", "machcontrol",
           "blowingcontrol", "mod_timedata", "dtnmod", "periodicity", "pvsqbc", "convolimpflow",
           "convolrcrflow", "incpbc", "lapackfuncs", "stats"]

_LU = {0: "LU_Fact ", 1: "forward ", 2: "backward", 3: "product "}


class _Obj:
    def __init__(self, p):
        self.p = p


def _F(flat, shape):
    """flat reference-layout array -> Fortran-ordered view of shape."""
    return np.asarray(flat, dtype=np.float64).reshape(shape, order="F")


class RefPhasta:
    def __init__(self, case, params: dict, root):
        root = Path(root)
        P = fexec.Program([root / "common", root / "compressible"])
        for f in SOURCES:
            P.load(root / f)
        P.stubs.update(timer=lambda *a: None, secs=lambda *a: 0.0, tmr=lambda *a: 0.0,
                       tmrc=lambda *a: 0.0, tnanq=lambda *a: None, rstat=lambda *a: None,
                       rstatcheck=lambda *a: None)
        N, E, Eb = case.nshg, case.nelem, case.nbelem
        self.N, self.case, self.params = N, case, dict(params)
        # interior blocks by topology: (connectivity, lcsyst, nshl, points)
        blocks = [(case.ien, 1, 4, 4), (getattr(case, "ienh", np.zeros((0, 8))), 2, 8, 8),
                  (getattr(case, "ienw", np.zeros((0, 6))), 3, 6, 6)]
        blocks = [b for b in blocks if len(b[0])]
        # boundary blocks (genbkb.f): the boundary tets, then each block of boundary hexes and
        # wedges as (connectivity, lcblkb lcsyst, nshl, nenbl, iBCB, BCB)
        bblocks = []
        if Eb:
            bblocks.append((case.ienb, 1, 4, 3, case.iBCB, case.BCB))
        for b in getattr(case, "bnd", []):
            bblocks.append((b.ien, 2 if b.lcsyst == 2 else 3, b.nshl, b.nshlb, b.iBCB, b.BCB))
        P.module("pointer_data", {
            "mien": [_Obj(np.asfortranarray(np.asarray(b[0]).astype(np.int64) + 1)) for b in blocks],
            "mmat": [_Obj(np.ones(len(b[0]), np.int64)) for b in blocks],
            "mxmudmi": [_Obj(np.zeros((len(b[0]), b[3]), order="F")) for b in blocks],
            "mienb": [_Obj(np.asfortranarray(np.asarray(b[0]).astype(np.int64) + 1)) for b in bblocks] or
                     [_Obj(np.zeros((1, 4), np.int64, order="F"))],
            "mmatb": [_Obj(np.ones(len(b[0]), np.int64)) for b in bblocks] or [_Obj(np.ones(1, np.int64))],
            "mibcb": [_Obj(np.asfortranarray(np.asarray(b[4]).astype(np.int64))) for b in bblocks] or
                     [_Obj(np.zeros((1, 2), np.int64, order="F"))],
            "mbcb": [_Obj(np.asfortranarray(np.asarray(b[5], dtype=np.float64))) for b in bblocks] or
                    [_Obj(np.zeros((1, 3, 6), order="F"))]})
        for m in MODULES:
            P.module(m, {})
        P.function("elmmfg")  # declares the COMMON blocks of common.h
        G = P.G
        T = json.loads((HERE / "tet_tables.json").read_text())
        TT = json.loads((HERE / "topo_tables.json").read_text())
        p = self.params
        G.numpe, G.myrank, G.master = 1, 0, 0
        G.numnp = G.nshg = N
        G.nshgt = N
        # numel counts the interior elements of every block (EGmass(numel, nedof, nedof) of SolGMRe)
        G.numel, G.numelb = E + case.nhex + case.nwedge, sum(len(b[0]) for b in bblocks)
        # nen is the largest element of the mesh (readnblk.f) and nedof = nflow*nshape (itrdrv.f:458)
        nenmax = max(nshl for _c, _l, nshl, _q in blocks)
        G.nen, G.ndof, G.nflow, G.nedof = nenmax, 5, 5, 5 * nenmax
        G.nshape = nenmax  # linear basis: nshape = nen (genint.f)
        G.ndofbc, G.ndibcb, G.ndbcb = 6, 2, 6
        G.nelblk, G.nelblb = len(blocks), len(bblocks)
        # lcblk(:,iblk): iel, lelCat, lcsyst, iorder, nenl, -, mattyp, ndofl, nsymdl, nshl
        iel = 1
        for ib, (con, lcsyst, nshl, _nq) in enumerate(blocks):
            G.lcblk[:, ib] = [iel, lcsyst, lcsyst, 1, nshl, 0, 1, 5, 0, nshl]
            iel += len(con)
        G.lcblk[0, len(blocks)] = iel
        # lcblkb(:,iblk): iel, lelCat, lcsyst, iorder, nenl, nenbl, mattyp, ndofl, nshl, nshlb
        iel = 1
        for ib, (con, lcsyst, nshl, nenbl, _ib, _b) in enumerate(bblocks):
            G.lcblkb[:, ib] = [iel, lcsyst, lcsyst, 1, nshl, nenbl, 1, 5, nshl, nenbl]
            iel += len(con)
        G.lcblkb[0, len(bblocks)] = iel
        G.nint[0], G.nintb[0] = 4, 3
        G.nint[1], G.nint[2] = 8, 6
        G.nintb[1], G.nintb[2], G.nintb[3] = 4, 3, 4   # genint.f: quad 2x2, wedge triangle 3, wedge quad 4
        G.qwt[0, :4] = T["Qwt"]
        G.qwt[1, :8] = TT["hex"]["Qwt"]
        G.qwt[2, :6] = TT["wedge"]["Qwt"]
        G.qwtb[0, :3] = T["Qwtb"]
        G.qwtb[1, :4] = TT["hex_quad_b"]["Qwtb"]
        G.qwtb[2, :3] = TT["wedge_tri_b"]["Qwtb"]
        G.qwtb[3, :4] = TT["wedge_quad_b"]["Qwtb"]
        G.datmat[0, 1, 0] = p["rmu"]
        G.pr, G.rgas, G.gamma, G.gamma1 = p["pr"], p["Rgas"], p["gamma"], p["gamma1"]
        G.dtgl, G.almi, G.alfi, G.gami = p["Dtgl"], p["almi"], p["alfi"], p["gami"]
        G.lhs, G.itau, G.ipord, G.idiff, G.isurf = 0, p["itau"], p["ipord"], p.get("idiff", 0), 0
        G.dtsfct, G.taucfct, G.temper = p["dtsfct"], p["taucfct"], p["temper"]
        G.ivart, G.navier, G.jactyp, G.idc = p["ivart"], p["Navier"], 0, p.get("iDC", 0)
        G.iremovestabtimeterm, G.entropypressure = p["iremoveStabTimeTerm"], p["EntropyPressure"]
        G.idflx = 12 if p.get("idiff", 0) >= 1 else 0  # (nflow-1)*nsd, solmfg.f:61-63
        G.kspace, G.ngmres, G.miniters = p["Kspace"], p["nGMRES"], p["minIters"]
        G.epstol[0] = p["etol"]
        G.etol = p["etol"]  # itrdrv.f:433
        G.epsm = p["epsM"]
        G.egmres = p["eGMRES"]
        G.iter, G.istep = p["iter"], p["istep"]
        G.iprec = 1
        G.ipred = 1  # input.config: Predictor at Start of Step = Same Velocity
        G.ntotgm = 0
        self.P, self.G = P, G
        self.shp = np.zeros((6, 32, 125), order="F")
        self.shgl = np.zeros((6, 3, 32, 125), order="F")
        self.shpb = np.zeros((6, 32, 125), order="F")
        self.shglb = np.zeros((6, 3, 32, 125), order="F")
        for q in range(4):
            self.shp[0, :4, q] = T["shp"][q]
            self.shgl[0, :, :4, q] = T["shgl"][q]
        for q in range(3):
            self.shpb[0, :4, q] = T["shpb"][q]
            self.shglb[0, :, :4, q] = T["shglb"][q]
        for top, (name, nq, nen) in ((1, ("hex", 8, 8)), (2, ("wedge", 6, 6))):
            for q in range(nq):
                self.shp[top, :nen, q] = TT[name]["shp"][q]
                self.shgl[top, :, :nen, q] = TT[name]["shgl"][q]
        # genshpb.f: shpb(lcsyst, :, q) for the boundary topologies 2, 3 and 4
        for top, (name, nq, nen) in ((1, ("hex_quad_b", 4, 8)), (2, ("wedge_tri_b", 3, 6)),
                                     (3, ("wedge_quad_b", 4, 6))):
            for q in range(nq):
                self.shpb[top, :nen, q] = TT[name]["shpb"][q]
                self.shglb[top, :, :nen, q] = TT[name]["shglb"][q]
        self.iBC = case.iBC.astype(np.int64)
        self.BC = np.asfortranarray(case.BC.T)
        self.iper = case.iper.astype(np.int64) + 1
        self.x = np.asfortranarray(case.x)
        self.ilwork = np.zeros(1, np.int64)
        self.rerr = np.zeros((N, 10), order="F")

    # ---- routines (flat reference layouts in and out)
    def ElmMFG(self, y, ac, iprec=1):
        N = self.N
        self.G.iprec = iprec
        yF, acF = _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5))
        res, rmes = np.zeros((N, 5), order="F"), np.zeros((N, 5), order="F")
        bd = np.zeros((N, 5, 5), order="F")
        self.P.call("elmmfg", yF, acF, self.x, self.shp, self.shgl, self.iBC, self.BC, self.shpb, self.shglb,
                    res, rmes, bd, self.iper, self.ilwork, self.rerr)
        self.G.iprec = 1
        return res.reshape(-1, order="F"), rmes.reshape(-1, order="F"), bd.reshape(-1, order="F")

    def ItrRes(self, yp, yc, ac, rmes):
        N = self.N
        rm = _F(np.array(rmes), (N, 5)).copy(order="F")
        self.P.call("itrres", _F(np.array(yp), (N, 5)), _F(np.array(yc), (N, 5)), self.x, self.shp, self.shgl,
                    self.iBC, self.BC, self.shpb, self.shglb, rm, self.iper, self.ilwork, _F(np.array(ac), (N, 5)))
        return rm.reshape(-1, order="F")

    def i3LU(self, bd, r, code):
        N = self.N
        bdF = _F(np.array(bd), (N, 5, 5)).copy(order="F")
        rF = _F(np.array(r), (N, 5)).copy(order="F") if r is not None else np.zeros((N, 5), order="F")
        self.P.call("i3lu", bdF, rF, _LU[code])
        return bdF.reshape(-1, order="F"), rF.reshape(-1, order="F")

    def itrBC(self, y, ac):
        N = self.N
        yF = _F(np.array(y), (N, 5)).copy(order="F")
        acF = _F(np.array(ac), (N, 5)).copy(order="F")
        self.P.call("itrbc", yF, acF, self.iBC, self.BC, self.iper, self.ilwork)
        return yF.reshape(-1, order="F"), acF.reshape(-1, order="F")

    def SolMFG(self, y, ac, yold, acold):
        N, K = self.N, self.params["Kspace"]
        G = self.G
        res = np.zeros((N, 5), order="F")
        bd = np.zeros((N, 5, 5), order="F")
        Dy = np.zeros((N, 5), order="F")
        HBrg = np.zeros((K + 1, K), order="F")
        eBrg, yBrg = np.zeros(K + 1), np.zeros(K)
        Rcos, Rsin = np.zeros(K), np.zeros(K)
        G.iprec = 1  # itrdrv.f:494 with LHSupd(1) = 1: the block diagonal is rebuilt every solve
        self.P.call("solmfg", _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5)), _F(np.array(yold), (N, 5)),
                    _F(np.array(acold), (N, 5)), self.x, self.iBC, self.BC, res, bd, HBrg, eBrg, yBrg, Rcos, Rsin,
                    self.iper, self.ilwork, self.shp, self.shgl, self.shpb, self.shglb, Dy, self.rerr)
        stats = {"iKs": int(G.iks), "lGMRES": int(G.lgmres), "ntotGM": int(G.ntotgm), "eGMRES": float(G.egmres),
                 "eBrg": eBrg.tolist()}
        return res.reshape(-1, order="F"), bd.reshape(-1, order="F"), Dy.reshape(-1, order="F"), stats

    def itrSetup(self, rho_inf: float, dt: float):
        """almi, alfi, gami, Dtgl of itrSetup (itrPC.f:6-46) for one time-sequence entry."""
        G = self.G
        G.itseq = 1
        G.rhoinf[0] = rho_inf
        G.delt[0] = dt
        y = np.zeros((self.N, 5), order="F")
        self.P.call("itrsetup", y, y.copy(order="F"))
        return {"almi": float(G.almi), "alfi": float(G.alfi), "gami": float(G.gami), "Dtgl": float(G.dtgl)}

    def itrPredict(self, yold, acold):
        N = self.N
        y, ac = np.zeros((N, 5), order="F"), np.zeros((N, 5), order="F")
        self.P.call("itrpredict", _F(np.array(yold), (N, 5)), _F(np.array(acold), (N, 5)), y, ac)
        return y.reshape(-1, order="F"), ac.reshape(-1, order="F")

    def itrCorrect(self, y, ac, yold, acold, Dy):
        N = self.N
        yF, acF = _F(np.array(y), (N, 5)).copy(order="F"), _F(np.array(ac), (N, 5)).copy(order="F")
        self.P.call("itrcorrect", yF, acF, _F(np.array(yold), (N, 5)), _F(np.array(acold), (N, 5)),
                    _F(np.array(Dy), (N, 5)))
        return yF.reshape(-1, order="F"), acF.reshape(-1, order="F")

    def itrUpdate(self, yold, acold, y, ac):
        N = self.N
        yoF, aoF = _F(np.array(yold), (N, 5)).copy(order="F"), _F(np.array(acold), (N, 5)).copy(order="F")
        self.P.call("itrupdate", yoF, aoF, _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5)))
        return yoF.reshape(-1, order="F"), aoF.reshape(-1, order="F")

    def time_step(self, yold, acold, nitr: int):
        """One step in the order of itrdrv.f:398-399, 427-634, 651-652 (matrix-free solve)."""
        y, ac = self.itrPredict(yold, acold)
        y, ac = self.itrBC(y, ac)
        iks = []
        for it in range(1, nitr + 1):
            self.G.iter = it
            _, _, Dy, st = self.SolMFG(y, ac, yold, acold)
            iks.append(st["iKs"])
            y, ac = self.itrCorrect(y, ac, yold, acold, Dy)
            y, ac = self.itrBC(y, ac)
        yold, acold = self.itrUpdate(yold, acold, y, ac)
        yold, acold = self.itrBC(yold, acold)
        return yold, acold, y, ac, iks

    # ---- assembled tangent (lhs = 1): the reference's default sparse solver
    def genadj(self, nnz: int = 40):
        """colm (nshg+1), rowp (icnt) of genadj.f: 1-based block CSR of the node adjacency."""
        N = self.N
        G = self.G
        G.nnz = nnz
        colm = np.zeros(N + 1, np.int64)
        rowp = np.zeros(N * nnz, np.int64)
        r = self.P.call("genadj", colm, rowp, 0)
        icnt = int(r[0])
        G.nnz_tot = icnt
        self.colm, self.rowp = colm, rowp
        return colm.copy(), rowp[:icnt].copy()

    def ElmGMRs(self, y, ac):
        """res, BDiag (from the tangent's diagonal blocks) and lhsK(25, nnz_tot) of ElmGMRs (lhs = 1)."""
        N = self.N
        G = self.G
        if not hasattr(self, "colm"):
            self.genadj()
        G.lhs, G.iprec = 1, 1
        lhsK = np.zeros((25, int(G.nnz_tot)), order="F")
        res, rmes = np.zeros((N, 5), order="F"), np.zeros((N, 5), order="F")
        bd = np.zeros((N, 5, 5), order="F")
        self.P.call("elmgmrs", _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5)), self.x, self.shp, self.shgl,
                    self.iBC, self.BC, self.shpb, self.shglb, res, rmes, bd, self.iper, self.ilwork, lhsK,
                    self.colm, self.rowp, self.rerr)
        G.lhs = 0
        return res.reshape(-1, order="F"), bd.reshape(-1, order="F"), lhsK

    def SolGMRs(self, y, ac, yold, acold):
        N, K = self.N, self.params["Kspace"]
        G = self.G
        if not hasattr(self, "colm"):
            self.genadj()
        G.lhs, G.iprec = 1, 1
        lhsK = np.zeros((25, int(G.nnz_tot)), order="F")
        res = np.zeros((N, 5), order="F")
        bd = np.zeros((N, 5, 5), order="F")
        Dy = np.zeros((N, 5), order="F")
        HBrg = np.zeros((K + 1, K), order="F")
        eBrg, yBrg = np.zeros(K + 1), np.zeros(K)
        Rcos, Rsin = np.zeros(K), np.zeros(K)
        self.P.call("solgmrs", _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5)), _F(np.array(yold), (N, 5)),
                    _F(np.array(acold), (N, 5)), self.x, self.iBC, self.BC, self.colm, self.rowp, lhsK, res, bd,
                    HBrg, eBrg, yBrg, Rcos, Rsin, self.iper, self.ilwork, self.shp, self.shgl, self.shpb,
                    self.shglb, Dy, self.rerr)
        G.lhs = 0
        # SolGMRs counts its cycles in lGMRESs (solgmr.f:511,526)
        stats = {"iKs": int(G.iks), "lGMRES": int(G.lgmress), "ntotGM": int(G.ntotgm)}
        return res.reshape(-1, order="F"), bd.reshape(-1, order="F"), Dy.reshape(-1, order="F"), lhsK, stats

    def Spsi3pre(self, lu, lhsK):
        """lhsK after Spsi3pre (spsi3pre.f:1) with the LU factors lu of i3LU."""
        N = self.N
        if not hasattr(self, "colm"):
            self.genadj()
        bdF = _F(np.array(lu), (N, 5, 5)).copy(order="F")
        out = np.array(lhsK, order="F", copy=True)
        self.P.call("spsi3pre", bdF, out, self.colm, self.rowp)
        return out

    def SparseAp(self, lhsK, p):
        """lhsK p of SparseAp (sparseap.f:1) with the periodic gather of p, then bc3per (solgmr.f:566)."""
        N = self.N
        if not hasattr(self, "colm"):
            self.genadj()
        pF = _F(np.array(p), (N, 5)).copy(order="F")
        self.P.call("sparseap", self.iper, self.ilwork, self.iBC, self.colm, self.rowp, np.asfortranarray(lhsK), pF)
        self.P.call("bc3per", self.iBC, pF, self.iper, self.ilwork, 5)
        return pF.reshape(-1, order="F")

    # ---- element-by-element solver (impl = 3x): EGmass(numel, nedof, nedof) stored per element
    def _egmass(self):
        G = self.G
        return np.zeros((int(G.numel), int(G.nedof), int(G.nedof)), order="F")

    def ElmGMRe(self, y, ac):
        """res, BDiag and the element tangents EGmass (after bc3LHS) of ElmGMRe (elmgmr.f:1)."""
        N = self.N
        G = self.G
        G.lhs, G.iprec = 1, 1
        EG = self._egmass()
        res, rmes = np.zeros((N, 5), order="F"), np.zeros((N, 5), order="F")
        bd = np.zeros((N, 5, 5), order="F")
        self.P.call("elmgmre", _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5)), self.x, self.shp, self.shgl,
                    self.iBC, self.BC, self.shpb, self.shglb, res, rmes, bd, self.iper, self.ilwork, EG, self.rerr)
        G.lhs = 0
        return res.reshape(-1, order="F"), bd.reshape(-1, order="F"), EG

    def i3pre(self, lu, EG):
        """EGmass after i3pre (i3pre.f:1) with the i3LU factors lu."""
        N = self.N
        bdF = _F(np.array(lu), (N, 5, 5)).copy(order="F")
        out = np.array(EG, order="F", copy=True)
        self.P.call("i3pre", bdF, np.zeros(1), out, self.ilwork)
        return out

    def Au1GMR(self, EG, p):
        """The element-by-element product of Au1GMR (au1gmr.f:1), then bc3per as SolGMRe applies it."""
        N = self.N
        pF = _F(np.array(p), (N, 5)).copy(order="F")
        self.P.call("au1gmr", np.asfortranarray(EG), pF, self.ilwork, self.iBC, self.iper)
        self.P.call("bc3per", self.iBC, pF, self.iper, self.ilwork, 5)
        return pF.reshape(-1, order="F")

    def SolGMRe(self, y, ac, yold, acold):
        N, K = self.N, self.params["Kspace"]
        G = self.G
        G.lhs, G.iprec = 1, 1
        EG = self._egmass()
        res = np.zeros((N, 5), order="F")
        bd = np.zeros((N, 5, 5), order="F")
        Dy = np.zeros((N, 5), order="F")
        HBrg = np.zeros((K + 1, K), order="F")
        eBrg, yBrg = np.zeros(K + 1), np.zeros(K)
        Rcos, Rsin = np.zeros(K), np.zeros(K)
        self.P.call("solgmre", _F(np.array(y), (N, 5)), _F(np.array(ac), (N, 5)), _F(np.array(yold), (N, 5)),
                    _F(np.array(acold), (N, 5)), self.x, self.iBC, self.BC, EG, res, bd, HBrg, eBrg, yBrg, Rcos,
                    Rsin, self.iper, self.ilwork, self.shp, self.shgl, self.shpb, self.shglb, Dy, self.rerr)
        G.lhs = 0
        stats = {"iKs": int(G.iks), "lGMRES": int(G.lgmres), "ntotGM": int(G.ntotgm)}
        return res.reshape(-1, order="F"), bd.reshape(-1, order="F"), Dy.reshape(-1, order="F"), EG, stats
