"""Generate tests/golden/ref_*.npz: outputs of the reference's own Fortran routines.

Runs where the reference tree is present (it reads the Fortran sources from
there).  fexec.py translates the reference's fixed-form sources of the hot
path into numpy code in memory and refrun.py sets the COMMON blocks, so the
arrays written here are what ElmMFG, ItrRes, i3LU, itrBC, SolMFG, itrSetup,
itrPredict, itrCorrect and itrUpdate of the reference compute for the seeded
inputs, which are stored beside the outputs; for the sparse solver (lhs = 1)
also genadj, ElmGMRs, Spsi3pre, SparseAp (with bc3per) and SolGMRs.

    python tests/golden/make_ref_golden.py [reference phSolver directory] [case names]
"""
from __future__ import annotations

import json
import sys
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(HERE), str(ROOT), str(ROOT / "tests")]

from helpers import channel, hexchannel, layered, mixed, vortex, wedgechannel  # noqa: E402
from refrun import RefPhasta  # noqa: E402

# the reference tree: $PHASTA_REFERENCE, else a directory "reference" beside the repository
DEFAULT_REF = Path(os.environ.get("PHASTA_REFERENCE", str(Path(__file__).resolve().parents[3] / "reference"))) / "phSolver"

# (name, case builder, parts): "elm" ElmMFG; "pieces" ItrRes, i3LU, itrBC; "solve" SolMFG;
# "step" itrSetup and one two-iteration time step; "sparse" genadj, ElmGMRs (assembled
# tangent lhsK), Spsi3pre, SparseAp and SolGMRs; "ebe" ElmGMRe (element tangents, stored as
# products with seeded probe vectors), i3pre, Au1GMR and SolGMRe -- on single-topology
# meshes only: with blocks of fewer nodes than the largest element, i3pre gathers BDiag
# through a section of its (numel, nshape, 5, 5) array into local's (npro, nshl, 25) dummy
# (i3pre.f), which scrambles the blocks of the smaller elements
ALL = ("elm", "pieces", "solve", "step")
CASES = [
    ("channel4", lambda: channel(4, ac_scale=0.05), ALL + ("sparse", "ebe")),
    ("vortex4", lambda: vortex(4), ALL + ("sparse", "ebe")),
    ("channel3_euler", lambda: channel(3, ac_scale=0.05, navier=0), ("elm",)),
    ("channel3_galerkin", lambda: channel(3, ac_scale=0.05, ivart=1), ("elm",)),
    # Kspace 3 with two cycles: the second cycle restarts from Au2MFG's R - J Dy
    # (SolGMRs restarts from its stale first vector: its test reads lGMRES, solgmr.f:528)
    ("channel4_restart", lambda: channel(4, ac_scale=0.05, Kspace=3, nGMRES=2), ("elm", "solve", "sparse", "ebe")),
    # tet, hex (lcsyst 2) and wedge (lcsyst 3) blocks
    ("mixed3", lambda: mixed(3, 3, (3, 3, 2)), ALL + ("sparse",)),
    # idiff = 1: the diffusive flux reconstructed (AsIq/e3q/qpbc) and its divergence in e3LS
    ("channel4_idiff", lambda: channel(4, ac_scale=0.05, idiff=1), ALL),
    ("mixed3_idiff", lambda: mixed(3, 3, (3, 3, 2), idiff=1), ("elm", "solve")),
    # single-topology hex and wedge meshes (periodic boxes)
    ("hex3", lambda: mixed(0, 3, 0), ("elm", "sparse", "ebe")),
    # discontinuity capturing: DC-mallet, DC-quadratic and DC-min (e3dc.f) on the matrix-free path
    ("channel4_dc1", lambda: channel(4, ac_scale=0.05, sigma=0.05, iDC=1), ("elm", "pieces", "solve")),
    ("channel4_dc2", lambda: channel(4, ac_scale=0.05, sigma=0.05, iDC=2), ("elm", "pieces")),
    ("channel4_dc3", lambda: channel(4, ac_scale=0.05, sigma=0.05, iDC=3), ("elm", "pieces")),
    ("mixed3_dc1", lambda: mixed(3, 3, (3, 3, 2), sigma=0.05, iDC=1), ("elm", "pieces")),
    # itau = 1: Diagonal-Franca tau (e3tau.f:54-139), matrix-free and assembled solvers
    ("channel4_tau1", lambda: channel(4, ac_scale=0.05, itau=1), ("elm", "pieces", "solve", "sparse")),
    ("mixed3_tau1", lambda: mixed(3, 3, (3, 3, 2), itau=1), ("elm", "pieces")),
    ("wedge3", lambda: mixed(0, 0, (3, 3, 2)), ("elm", "sparse", "ebe")),
    # one connected mesh whose hex, prism and tet layers share their interface nodes: every
    # interface node sums contributions of two element topologies
    ("layered3", lambda: layered(3, (2, 1, 2)), ALL + ("sparse",)),
    ("layered3_idiff", lambda: layered(3, (1, 1, 1), idiff=1), ("elm", "solve")),
    # boundary hexes and wedges (AsBMFG/e3b with lcsyst 2, 3 and 4): inflow and outflow through
    # hex faces; through prism quadrilaterals, with prism triangles on the z walls; and the
    # connected layered mesh with tet, hex and prism faces on its inflow and outflow planes
    ("hexchannel3", lambda: hexchannel(3), ALL + ("sparse",)),
    ("wedgechannel3", lambda: wedgechannel((3, 3, 2)), ("elm", "pieces", "solve")),
    ("layered3_open", lambda: layered(3, (2, 1, 2), periodic_x=False), ALL + ("sparse",)),
]


def _params_json(p):
    return json.dumps({k: (float(v) if isinstance(v, float) else v) for k, v in p.items()}, sort_keys=True)


def make(name, build, parts, ref_root):
    case, p, y, ac = build()
    R = RefPhasta(case, p, ref_root)
    out = {"params": np.array(_params_json(p)), "nshg": np.array(case.nshg), "nelem": np.array(case.nelem),
           "ien": case.ien.astype(np.int32), "x": case.x_ref(), "y": y, "ac": ac}
    res, rmes, bd = R.ElmMFG(y, ac)
    out.update(elm_res=res, elm_rmes=rmes, elm_bd=bd)
    if "pieces" in parts:
        rng = np.random.default_rng(7)
        yp = y * (1.0 + 1e-3 * rng.standard_normal(y.shape))
        r0 = rng.standard_normal(y.shape)
        out.update(yp=yp, r0=r0, itrres_rmes=R.ItrRes(yp, y, ac, r0))
        lu, _ = R.i3LU(bd, None, 0)
        out["lu_fact"] = lu
        for code, key in ((1, "lu_forward"), (2, "lu_backward"), (3, "lu_product")):
            out[key] = R.i3LU(lu, r0, code)[1]
        yb, ab = R.itrBC(yp, ac)
        out.update(itrbc_y=yb, itrbc_ac=ab)
    if "solve" in parts:
        sres, sbd, sDy, st = R.SolMFG(y, ac, y, ac)
        out.update(sol_res=sres, sol_bd=sbd, sol_Dy=sDy, sol_iKs=np.array(st["iKs"]),
                   sol_lGMRES=np.array(st["lGMRES"]), sol_ntotGM=np.array(st["ntotGM"]),
                   sol_eGMRES=np.array(st["eGMRES"]))
    if "step" in parts:
        rho_inf = 0.5
        setup = R.itrSetup(rho_inf, 1.0 / p["Dtgl"])
        out["setup"] = np.array([setup[k] for k in ("almi", "alfi", "gami", "Dtgl")])
        R2 = RefPhasta(case, p, ref_root)
        yold, acold, y1, ac1, iks = R2.time_step(y, ac, 2)
        out.update(step_yold=yold, step_acold=acold, step_y=y1, step_ac=ac1, step_iks=np.array(iks))
    if "sparse" in parts:
        R3 = RefPhasta(case, p, ref_root)  # fresh COMMON: lGMRES = ntotGM = 0
        colm, rowp = R3.genadj()
        gres, gbd, lhsK = R3.ElmGMRs(y, ac)
        out.update(sp_colm=colm.astype(np.int32), sp_rowp=rowp.astype(np.int32), sp_lhsK=lhsK, sp_res=gres,
                   sp_bd=gbd)
        # Spsi3pre with the LU factors of the golden BDiag, then SparseAp on a seeded vector
        lu, _ = R3.i3LU(gbd, None, 0)
        pre = R3.Spsi3pre(lu, lhsK)
        rng = np.random.default_rng(11)
        pv = rng.standard_normal(5 * case.nshg)
        out.update(sp_lu=lu, sp_pre=pre, sp_p=pv, sp_ap=R3.SparseAp(pre, pv))
        R4 = RefPhasta(case, p, ref_root)
        R4.genadj()
        # (its preconditioned lhsK equals sp_pre bit for bit, so it is not stored again)
        sres, sbd, sDy, _, st = R4.SolGMRs(y, ac, y, ac)
        out.update(sps_res=sres, sps_bd=sbd, sps_Dy=sDy, sps_iKs=np.array(st["iKs"]),
                   sps_lGMRES=np.array(st["lGMRES"]), sps_ntotGM=np.array(st["ntotGM"]))
    if "ebe" in parts:
        R5 = RefPhasta(case, p, ref_root)
        eres, ebd, EG = R5.ElmGMRe(y, ac)
        rng = np.random.default_rng(13)
        v = rng.standard_normal(EG.shape[:2])
        lu, _ = R5.i3LU(ebd, None, 0)
        pre = R5.i3pre(lu, EG)
        pv = rng.standard_normal(5 * case.nshg)
        out.update(ebe_res=eres, ebe_bd=ebd, ebe_v=v, ebe_EGv=np.einsum("eij,ej->ei", EG, v), ebe_lu=lu,
                   ebe_prev=np.einsum("eij,ej->ei", pre, v), ebe_p=pv, ebe_ap=R5.Au1GMR(pre, pv))
        R6 = RefPhasta(case, p, ref_root)
        sres, sbd, sDy, _, st = R6.SolGMRe(y, ac, y, ac)
        out.update(ebe_sres=sres, ebe_sbd=sbd, ebe_Dy=sDy, ebe_iKs=np.array(st["iKs"]),
                   ebe_lGMRES=np.array(st["lGMRES"]), ebe_ntotGM=np.array(st["ntotGM"]))
    path = HERE / f"ref_{name}.npz"
    np.savez_compressed(path, **out)
    print(f"{path.name}: {path.stat().st_size // 1024} KiB, nshg {case.nshg}, nelem {case.nelem}")


def main():
    ref_root = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF
    if not (ref_root / "compressible" / "e3.f").exists():
        raise SystemExit(f"reference sources not found under {ref_root}")
    only = set(sys.argv[2:])
    for name, build, parts in CASES:
        if not only or name in only:
            make(name, build, parts, ref_root)


if __name__ == "__main__":
    main()
