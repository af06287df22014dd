"""Host-side mirror of PHASTA's compressible hot-path routines on the GPU.

``GpuSolver`` owns one GPU context (``phgpu_ctx``) created from a mesh and the
COMMON-block parameters; its methods carry the reference routine names and
argument meaning (arrays in the reference layout, see include/phgpu.h):

    ElmMFG(y, ac)                -> res, rmes, BDiag          elmmfg.f:1
    ElmRes(y, ac)                -> res                       (ElmMFG with ires = 1)
    ItrRes(yp, yc, ac, rmes)     -> rmes (accumulated)        itrres.f:1
    i3LU(BDiag, r, code)                                      i3lu.f:1
    SolMFG(y, ac)                -> res, BDiag, Dy, stats     solmfg.f:1
    itrCorrect(y, ac, yold, acold, Dy)                        itrPC.f:128 + itrbc.f
    newton(y, ac, yold, acold)   one flow solve of itrdrv      itrdrv.f:489-598
    time_step(yold, acold, nitr) itrPredict + nitr solves + itrUpdate

and the sparse solver of the reference's impl = 1x path (lhs = 1):

    genadj(case, nnz)            -> colm, rowp (1-based)      genadj.f:1 (host only)
    ElmGMRs(y, ac)               -> res, BDiag, lhsK          elmgmr.f:280
    Spsi3pre(lu, lhsK)           -> lhsK                      spsi3pre.f:1
    SparseAp(lhsK, p)            -> lhsK p (+ bc3per)         sparseap.f:1, bc3per.f:1
    SolGMRs(y, ac, lhs)          -> res, BDiag, Dy, lhsK, st  solgmr.f:480

and the element-by-element solver (impl = 3x; one element topology):

    ElmGMRe(y, ac)               -> res, BDiag, EGmass        elmgmr.f:1
    i3pre(lu, EGmass)            -> EGmass                    i3pre.f:1
    Au1GMR(EGmass, p)            -> sum_e EGmass_e p (+bc3per) au1gmr.f:1
    SolGMRe(y, ac)               -> res, BDiag, Dy, EGmass, st solgmr.f:1

lhsK is returned as an (nnz_tot, 25) array: row k is the reference's lhsK(:, k); EGmass as
an (numel, nedof, nedof) array view of the reference's EGmass.

Every call runs on the GPU; a non-zero status from the library raises
``PhgpuError`` (the reference would stop in error()/tnanq).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .mesh import GAMMA, GAMMA1, Case, rgas, time_params


class PhgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"phgpu status {code} ({L.STATUS.get(code, '?')}): {msg}")
        self.code = code


def make_params(mu: float, dt: float, rho_inf: float = 0.5, Kspace: int = 10, etol: float = 1e-3,
                minIters: int = 1, nGMRES: int = 1, pr: float = 0.72, precision: int = L.PHGPU_FP64,
                ap_mode: int = L.PHGPU_AP_FD, navier: int = 1, ivart: int = 2,
                outer_residual: int = L.PHGPU_RES_FP64, idiff: int = 0, iDC: int = 0, itau: int = 0,
                precond: int = L.PHGPU_PRECOND_BDIAG) -> dict:
    """The COMMON-block values of the hot path (input.config defaults otherwise)."""
    p = {"Rgas": rgas(), "gamma": GAMMA, "gamma1": GAMMA1, "pr": pr, "rmu": mu,
         "dtsfct": 1.0, "taucfct": 1.0, "temper": 1.0, "itau": itau, "ivart": ivart,
         "iremoveStabTimeTerm": 0, "Navier": navier, "ipord": 1, "EntropyPressure": 0,
         "Kspace": Kspace, "nGMRES": nGMRES, "minIters": minIters, "etol": etol,
         "epsM": float(np.sqrt(np.finfo(np.float64).eps)), "eGMRES": 0.0, "iter": 1, "istep": 0,
         "precision": precision, "ap_mode": ap_mode, "outer_residual": outer_residual, "idiff": idiff,
         "iDC": iDC, "precond": precond}
    p.update(time_params(rho_inf, dt))
    return p


def _config(p: dict) -> L.Config:
    c = L.Config()
    for name, _ in L.Config._fields_:
        if name in p:
            setattr(c, name, p[name])
    return c


@dataclass
class SolveStats:
    iKs: int
    lGMRES: int
    ntotGM: int
    unorm0: float
    echeck: float
    eGMRES: float
    totres: float
    rnorm: float
    t_assembly_ms: float
    t_gmres_ms: float
    net_its: int = 0
    net_fallback: int = L.PHGPU_NET_PLAIN


def _stats(s: L.Stats) -> SolveStats:
    return SolveStats(s.iKs, s.lGMRES, s.ntotGM, s.unorm0, s.echeck, s.eGMRES, s.totres, s.rnorm,
                      s.t_assembly_ms, s.t_gmres_ms, s.net_its, s.net_fallback)


class _MeshArrays:
    """The phgpu_mesh of a Case, with the host arrays it points to kept alive."""

    def __init__(self, case: Case):
        self.x = case.x_ref()
        self.ien = np.ascontiguousarray(case.ien, dtype=np.int32).reshape(-1)
        self.ienb = np.ascontiguousarray(case.ienb, dtype=np.int32).reshape(-1)
        self.iBCB = np.ascontiguousarray(case.iBCB, dtype=np.int32).reshape(-1)
        self.BCB = np.ascontiguousarray(case.BCB, dtype=np.float64).reshape(-1)
        self.iBC = np.ascontiguousarray(case.iBC, dtype=np.int32)
        self.BC = np.ascontiguousarray(case.BC, dtype=np.float64).reshape(-1)
        self.iper = np.ascontiguousarray(case.iper, dtype=np.int32)
        self.ienh = np.ascontiguousarray(case.ienh, dtype=np.int32).reshape(-1)
        self.ienw = np.ascontiguousarray(case.ienw, dtype=np.int32).reshape(-1)
        nb = case.nbelem
        bnd = getattr(case, "bnd", [])
        self.bnd = [(np.ascontiguousarray(b.ien, dtype=np.int32).reshape(-1),
                     np.ascontiguousarray(b.iBCB, dtype=np.int32).reshape(-1),
                     np.ascontiguousarray(b.BCB, dtype=np.float64).reshape(-1)) for b in bnd]
        self.bblk = (L.BndBlock * max(1, len(bnd)))(
            *[L.BndBlock(b.lcsyst, b.ien.shape[0], L.iptr(a[0]), L.iptr(a[1]), L.dptr(a[2]))
              for b, a in zip(bnd, self.bnd)])
        self.m = L.Mesh(case.nshg, case.nelem, L.iptr(self.ien) if case.nelem else None, L.dptr(self.x), nb,
                        L.iptr(self.ienb) if nb else None, L.iptr(self.iBCB) if nb else None,
                        L.dptr(self.BCB) if nb else None, L.iptr(self.iBC), L.dptr(self.BC), L.iptr(self.iper),
                        case.nhex, L.iptr(self.ienh) if case.nhex else None, case.nwedge,
                        L.iptr(self.ienw) if case.nwedge else None, len(bnd), self.bblk if bnd else None)


def genadj(case: Case, nnz: int = 40):
    """genadj.f: colm (nshg+1) and rowp (nnz_tot), 1-based; runs on the host (no GPU)."""
    lib = L.lib()
    ma = _MeshArrays(case)
    colm = np.zeros(case.nshg + 1, np.int32)
    rowp = np.zeros(case.nshg * nnz, np.int32)
    icnt = C.c_int()
    rc = lib.phgpu_genadj(C.byref(ma.m), nnz, L.iptr(colm), L.iptr(rowp), C.byref(icnt))
    if rc != 0:
        raise PhgpuError(rc, "genadj: more than nnz blocks in a row" if rc == L.PHGPU_ERR_TOO_LARGE else "genadj")
    return colm, rowp[: icnt.value].copy()


def rcm_order(case: Case) -> tuple[np.ndarray, int, int]:
    """Reverse Cuthill-McKee node order (phgpu_rcm_order, host only): new_of_old and the graph's
    bandwidth before and after; apply it with mesh.renumber / mesh.renumber_field."""
    lib = L.lib()
    ma = _MeshArrays(case)
    p = np.zeros(case.nshg, np.int32)
    b0, b1 = C.c_longlong(), C.c_longlong()
    rc = lib.phgpu_rcm_order(C.byref(ma.m), L.iptr(p), C.byref(b0), C.byref(b1))
    if rc != 0:
        raise PhgpuError(rc, "rcm_order: invalid mesh")
    return p, b0.value, b1.value


class GpuSolver:
    def __init__(self, case: Case, params: dict):
        self.lib = L.lib()
        self.case = case
        self.params = dict(params)
        self.nshg = case.nshg
        self._mesh = _MeshArrays(case)  # kept alive for the duration of create
        m = self._mesh.m
        self._cfg = _config(self.params)
        h = C.c_void_p()
        rc = self.lib.phgpu_create(C.byref(m), C.byref(self._cfg), C.byref(h))
        if rc != 0:
            raise PhgpuError(rc, "phgpu_create failed")
        self.h = h
        self.ntotGM = 0

    # -- helpers --
    def close(self):
        if getattr(self, "h", None):
            self.lib.phgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise PhgpuError(rc, self.lib.phgpu_last_error(self.h).decode())

    def set_params(self, **kw):
        """Change COMMON-block values; the library-managed ones (eGMRES, iter,
        istep) keep their current device-side values unless given here."""
        cur = self.get_params()
        cur.update(kw)
        self.params.update(cur)
        self._cfg = _config(self.params)
        self._check(self.lib.phgpu_set_config(self.h, C.byref(self._cfg)))

    def get_params(self) -> dict:
        c = L.Config()
        self._check(self.lib.phgpu_get_config(self.h, C.byref(c)))
        return {name: getattr(c, name) for name, _ in L.Config._fields_}

    def _v(self, k: int = 5) -> np.ndarray:
        return np.zeros(k * self.nshg, dtype=np.float64)

    @property
    def num_colors(self) -> int:
        return self.lib.phgpu_num_colors(self.h)

    @property
    def kernel_launches(self) -> int:
        return self.lib.phgpu_kernel_launches(self.h)

    @property
    def graph_cycles(self) -> int:
        """GMRES cycles run as one CUDA graph (-1: the graph could not be built)."""
        return self.lib.phgpu_graph_cycles(self.h)

    @property
    def step_graphs(self) -> int:
        """Time steps run as one CUDA graph (-1: the graph could not be built)."""
        return self.lib.phgpu_step_graphs(self.h)

    def set_tuning(self, lin_minb: int = 0, ress_minb: int = 0) -> None:
        """Force the pipelined sweeps' variants (minimum CTAs per SM: linearized product 3 or 4,
        split residual 2, 3 or 4), or with (0, 0) return to autotuning at the next solve, or with
        (-1, -1) autotune timing every variant whatever the mesh size."""
        self._check(self.lib.phgpu_set_tuning(self.h, int(lin_minb), int(ress_minb)))

    def tuning(self) -> dict:
        """The sweep variants in use, how they were chosen and each variant's tuned time (ms)."""
        lm, rm = C.c_int(0), C.c_int(0)
        ms = np.zeros(5)
        state = self.lib.phgpu_tuning(self.h, C.byref(lm), C.byref(rm), L.dptr(ms))
        how = {0: "default", 1: "tuned", 2: "forced"}[state]
        return {"lin_minb": lm.value, "ress_minb": rm.value, "how": how,
                "lin_ms": {3: ms[0], 4: ms[1]}, "ress_ms": {2: ms[2], 3: ms[3], 4: ms[4]}}

    def stream(self) -> int:
        return self.lib.phgpu_stream(self.h)

    # -- reference routines --
    def ElmMFG(self, y, ac, iprec: int = 1):
        res, rmes = self._v(), self._v()
        bd = self._v(25) if iprec else None
        self._check(self.lib.phgpu_elmmfg(self.h, L.dptr(y), L.dptr(ac), L.dptr(res), L.dptr(rmes),
                                          L.dptr(bd), iprec))
        return res, rmes, bd

    def ElmRes(self, y, ac):
        res = self._v()
        self._check(self.lib.phgpu_elmres(self.h, L.dptr(y), L.dptr(ac), L.dptr(res)))
        return res

    def ItrRes(self, yp, yc, ac, rmes=None):
        rmes = self._v() if rmes is None else np.array(rmes, dtype=np.float64)
        self._check(self.lib.phgpu_itrres(self.h, L.dptr(yp), L.dptr(yc), L.dptr(ac), L.dptr(rmes)))
        return rmes

    def i3LU(self, bdiag, r, code):
        bdiag = np.array(bdiag, dtype=np.float64)
        r = None if r is None else np.array(r, dtype=np.float64)
        self._check(self.lib.phgpu_i3lu(self.h, L.dptr(bdiag), L.dptr(r), code))
        return bdiag, r

    def SolMFG(self, y, ac):
        res, bd, Dy = self._v(), self._v(25), self._v()
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_solmfg(self.h, L.dptr(y), L.dptr(ac), L.dptr(res), L.dptr(bd), L.dptr(Dy),
                                          C.byref(st)))
        self.ntotGM = st.ntotGM
        return res, bd, Dy, _stats(st)

    def itrCorrect(self, y, ac, yold, acold, Dy):
        y, ac = np.array(y, dtype=np.float64), np.array(ac, dtype=np.float64)
        self._check(self.lib.phgpu_itrcorrect(self.h, L.dptr(y), L.dptr(ac), L.dptr(yold), L.dptr(acold), L.dptr(Dy)))
        return y, ac

    def newton(self, y, ac, yold, acold):
        y, ac = np.array(y, dtype=np.float64), np.array(ac, dtype=np.float64)
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_newton(self.h, L.dptr(y), L.dptr(ac), L.dptr(yold), L.dptr(acold), C.byref(st)))
        self.ntotGM = st.ntotGM
        return y, ac, _stats(st)

    def time_step(self, yold, acold, nitr: int):
        yold, acold = np.array(yold, dtype=np.float64), np.array(acold, dtype=np.float64)
        y, ac = self._v(), self._v()
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_time_step(self.h, L.dptr(yold), L.dptr(acold), L.dptr(y), L.dptr(ac), nitr,
                                             C.byref(st)))
        self.ntotGM = st.ntotGM
        return yold, acold, y, ac, _stats(st)

    # -- sparse solver (lhs = 1) --
    @property
    def nnz_tot(self) -> int:
        n = C.c_int()
        self._check(self.lib.phgpu_nnz_tot(self.h, C.byref(n)))
        return n.value

    def ElmGMRs(self, y, ac):
        res, bd = self._v(), self._v(25)
        lhsK = np.zeros((self.nnz_tot, 25))
        self._check(self.lib.phgpu_elmgmrs(self.h, L.dptr(y), L.dptr(ac), L.dptr(res), L.dptr(bd), L.dptr(lhsK)))
        return res, bd, lhsK

    def Spsi3pre(self, lu, lhsK):
        out = np.array(lhsK, dtype=np.float64, order="C")
        self._check(self.lib.phgpu_spsi3pre(self.h, L.dptr(np.ascontiguousarray(lu, dtype=np.float64)), L.dptr(out)))
        return out

    def SparseAp(self, lhsK, p):
        p = np.array(p, dtype=np.float64)
        self._check(self.lib.phgpu_sparseap(self.h, L.dptr(np.ascontiguousarray(lhsK, dtype=np.float64)), L.dptr(p)))
        return p

    def SolGMRs(self, y, ac, lhs: int = 1, lGMRES_common: int = 0):
        """SolGMRs; lGMRES_common is the COMMON lGMRES its restart test reads (solgmr.f:528)."""
        res, bd, Dy = self._v(), self._v(25), self._v()
        lhsK = np.zeros((self.nnz_tot, 25)) if self.params.get("precision", L.PHGPU_FP64) == L.PHGPU_FP64 else None
        st = L.Stats()
        st.ntotGM = self.ntotGM
        st.lGMRES = lGMRES_common
        self._check(self.lib.phgpu_solgmrs(self.h, L.dptr(y), L.dptr(ac), lhs, L.dptr(res), L.dptr(bd), L.dptr(Dy),
                                           L.dptr(lhsK), C.byref(st)))
        self.ntotGM = st.ntotGM
        return res, bd, Dy, lhsK, _stats(st)

    # -- element-by-element solver (one element topology) --
    def _eg(self):
        c = self.case
        n = c.nelem + c.nhex + c.nwedge
        nd = 20 if c.nelem else 40 if c.nhex else 30
        return np.zeros((nd, nd, n))  # C order (j, i, e): the reference's EGmass(e, i, j)

    def ElmGMRe(self, y, ac):
        res, bd, EG = self._v(), self._v(25), self._eg()
        self._check(self.lib.phgpu_elmgmre(self.h, L.dptr(y), L.dptr(ac), L.dptr(res), L.dptr(bd), L.dptr(EG)))
        return res, bd, EG.transpose(2, 1, 0)

    def i3pre(self, lu, EG):
        out = np.ascontiguousarray(np.asarray(EG).transpose(2, 1, 0))
        self._check(self.lib.phgpu_i3pre(self.h, L.dptr(np.ascontiguousarray(lu, dtype=np.float64)), L.dptr(out)))
        return out.transpose(2, 1, 0)

    def Au1GMR(self, EG, p):
        p = np.array(p, dtype=np.float64)
        eg = np.ascontiguousarray(np.asarray(EG).transpose(2, 1, 0))
        self._check(self.lib.phgpu_au1gmr(self.h, L.dptr(eg), L.dptr(p)))
        return p

    def SolGMRe(self, y, ac):
        res, bd, Dy = self._v(), self._v(25), self._v()
        EG = self._eg() if self.params.get("precision", L.PHGPU_FP64) == L.PHGPU_FP64 else None
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_solgmre(self.h, L.dptr(y), L.dptr(ac), L.dptr(res), L.dptr(bd), L.dptr(Dy),
                                           L.dptr(EG), C.byref(st)))
        self.ntotGM = st.ntotGM
        return res, bd, Dy, (None if EG is None else EG.transpose(2, 1, 0)), _stats(st)

    def time_step_into(self, yold, acold, y, ac, nitr: int):
        """time_step on caller-owned arrays (float64, contiguous; pinned host memory keeps the
        copies at the link's bandwidth): yold/acold updated in place, y/ac written."""
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_time_step(self.h, L.dptr(yold), L.dptr(acold), L.dptr(y), L.dptr(ac), nitr,
                                             C.byref(st)))
        self.ntotGM = st.ntotGM
        return _stats(st)

    # -- device-resident path (benchmarks) --
    def upload(self, y=None, ac=None, yold=None, acold=None):
        self._check(self.lib.phgpu_upload_state(self.h, L.dptr(y), L.dptr(ac), L.dptr(yold), L.dptr(acold)))

    def download(self):
        y, ac, yo, ao = self._v(), self._v(), self._v(), self._v()
        self._check(self.lib.phgpu_download_state(self.h, L.dptr(y), L.dptr(ac), L.dptr(yo), L.dptr(ao)))
        return y, ac, yo, ao

    def newton_dev(self) -> SolveStats:
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_newton_dev(self.h, C.byref(st)))
        self.ntotGM = st.ntotGM
        return _stats(st)

    def time_step_dev(self, nitr: int) -> SolveStats:
        st = L.Stats()
        st.ntotGM = self.ntotGM
        self._check(self.lib.phgpu_time_step_dev(self.h, nitr, C.byref(st)))
        self.ntotGM = st.ntotGM
        return _stats(st)

    def set_bc(self, BC):
        """New Dirichlet values BC(nshg, 6) (the reference passes BC to every ElmMFG/SolMFG call)."""
        bc = np.ascontiguousarray(BC, dtype=np.float64).reshape(-1)
        self._check(self.lib.phgpu_set_bc(self.h, L.dptr(bc)))

    # -- learned preconditioner (flexible GMRES with a message-passing network; no reference
    #    counterpart: the reference's preconditioner is the block-diagonal LU of i3lu.f) --
    def net_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self.lib.phgpu_net_set_weights(self.h, L.fptr(w), w.size))

    def net_get_weights(self) -> np.ndarray:
        w = np.zeros(L.PHGPU_NET_NPARAM, np.float32)
        self._check(self.lib.phgpu_net_get_weights(self.h, L.fptr(w), w.size))
        return w

    def net_graph(self):
        """(nstart (nshg+1), nbr (nnz, neighbour | shift code << 26), geo [Lx, Ly, Lz, 1/hbar])."""
        nnz = C.c_longlong()
        geo = np.zeros(4, np.float32)
        self._check(self.lib.phgpu_net_graph(self.h, None, None, 0, C.byref(nnz), L.fptr(geo)))
        nstart = np.zeros(self.nshg + 1, np.int32)
        nbr = np.zeros(max(nnz.value, 1), np.uint32)
        self._check(self.lib.phgpu_net_graph(self.h, L.iptr(nstart), nbr.ctypes.data_as(C.POINTER(C.c_uint)),
                                             nbr.size, C.byref(nnz), L.fptr(geo)))
        return nstart, nbr[: nnz.value], geo

    def net_usage(self) -> dict:
        """Solves with the learned preconditioner selected, by outcome, and whether it is switched off."""
        c = (C.c_longlong * 4)()
        self._check(self.lib.phgpu_net_usage(self.h, c))
        return {"used": c[0], "fell_back": c[1], "plain": c[2], "off": bool(c[3])}

    def net_features(self) -> np.ndarray:
        out = np.zeros((self.nshg, 32), np.float32)
        self._check(self.lib.phgpu_net_features(self.h, L.fptr(out)))
        return out

    def net_apply(self, v, hidden: bool = False):
        """z = P(v) (res layout); with hidden, also h0..h3 (4, nshg, 64) and the decoder outputs (nshg, 8)."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        z = np.zeros_like(v)
        hb = np.zeros((4, self.nshg, 64), np.float32) if hidden else None
        ob = np.zeros((self.nshg, 8), np.float32) if hidden else None
        self._check(self.lib.phgpu_net_apply(self.h, L.dptr(v), L.dptr(z), L.fptr(hb), L.fptr(ob)))
        return (z, hb, ob) if hidden else z

    def net_loss_grad(self, v, t):
        v = np.ascontiguousarray(v, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        loss = C.c_double()
        grad = np.zeros(L.PHGPU_NET_NPARAM, np.float32)
        self._check(self.lib.phgpu_net_loss_grad(self.h, L.dptr(v), L.dptr(t), C.byref(loss), L.fptr(grad)))
        return loss.value, grad

    def net_pairs(self, cap: int):
        self._check(self.lib.phgpu_net_pairs(self.h, cap))

    def net_collect(self, slot: int, which: int = 0):
        """Training pair from the last solve: its solution (which = 0) or Krylov vector ``which``."""
        self._check(self.lib.phgpu_net_collect(self.h, slot, which))

    def net_train(self, epochs: int, lr: float = 1e-3, npairs: int = 0, clip: float = 1.0, seed: int = 1,
                  renormalize: bool = True, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> dict:
        cfg = L.NetTrainConfig(epochs, npairs, lr, beta1, beta2, eps, clip, seed, 1 if renormalize else 0)
        st = L.NetTrainStats()
        self._check(self.lib.phgpu_net_train(self.h, C.byref(cfg), C.byref(st)))
        return {"loss_first": st.loss_first, "loss_last": st.loss_last, "ms": st.ms, "steps": st.steps}

    def residual_norm_dev(self) -> float:
        r = C.c_double()
        self._check(self.lib.phgpu_residual_norm_dev(self.h, C.byref(r)))
        return r.value

    def sweep_dev(self, which: int):
        self._check(self.lib.phgpu_sweep_dev(self.h, which))
