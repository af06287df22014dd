"""The CPU oracle against golden vectors computed by the reference's own Fortran.

tests/golden/ref_*.npz hold the outputs of the reference routines (ElmMFG,
ItrRes, i3LU, itrBC, SolMFG, itrSetup, itrPredict/itrCorrect/itrUpdate and one
two-iteration time step in the order of itrdrv.f), executed from the reference
sources by tests/golden/make_ref_golden.py, with the seeded inputs they were
run on.  Tolerances (relative 2-norm):
  * element routines, LU, boundary conditions: 1e-12 (operation order differs
    from the Fortran array syntax only in the last bits);
  * SolMFG: the same Krylov iteration count, eGMRES within 1e-2 and Dy within
    1e-5: itrFDI divides a second difference of residuals by epsM, so a one-ulp
    change of the state moves eGMRES by up to ~0.4% and, through Au1MFG, Dy by
    ~2e-6 on these cases;
  * time step: y within 1e-9, ac within 1e-7 (the state moves by the
    finite-difference Dy above, ac by Dtgl/gami times it).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import rel
from oracle import pyoracle

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from make_ref_golden import CASES  # noqa: E402

FIXTURES = {name: (build, parts) for name, build, parts in CASES}


def having(part):
    return [n for n, (_, parts) in FIXTURES.items() if part in parts]


def load(name):
    path = GOLDEN / f"ref_{name}.npz"
    d = dict(np.load(path, allow_pickle=False))
    build, _parts = FIXTURES[name]
    case, p, y, ac = build()
    assert np.array_equal(d["ien"], case.ien.astype(np.int32)), "mesh generator changed"
    assert np.array_equal(d["x"], case.x_ref())
    assert np.array_equal(d["y"], y) and np.array_equal(d["ac"], ac), "seeded state changed"
    stored = json.loads(str(d["params"]))
    stored.setdefault("iDC", 0)  # fixtures written before the option hold no key for it (it was off)
    stored.setdefault("precond", 0)  # likewise: the block-diagonal preconditioner of the reference
    assert stored == json.loads(json.dumps(p, sort_keys=True))
    return d, case, p


@pytest.mark.parametrize("name", list(FIXTURES))
def test_oracle_elmmfg_matches_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    r, m, b = o.ElmMFG(d["y"], d["ac"])
    assert rel(r, d["elm_res"]) < 1e-12
    assert rel(m, d["elm_rmes"]) < 1e-12
    assert rel(b, d["elm_bd"]) < 1e-12


@pytest.mark.parametrize("name", having("pieces"))
def test_oracle_itrres_lu_itrbc_match_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    assert rel(o.ItrRes(d["yp"], d["y"], d["ac"], d["r0"]), d["itrres_rmes"]) < 1e-12
    lu, _ = o.i3LU(d["elm_bd"], None, 0)
    assert rel(lu, d["lu_fact"]) < 1e-12
    for code, key in ((1, "lu_forward"), (2, "lu_backward"), (3, "lu_product")):
        assert rel(o.i3LU(d["lu_fact"], d["r0"], code)[1], d[key]) < 1e-12, key
    yb, ab = o.itrBC(d["yp"], d["ac"])
    assert rel(yb, d["itrbc_y"]) < 1e-15 and rel(ab, d["itrbc_ac"]) < 1e-15


@pytest.mark.parametrize("name", having("solve"))
def test_oracle_solmfg_matches_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    res, bd, Dy, st = o.SolMFG(d["y"], d["ac"])
    assert rel(res, d["sol_res"]) < 1e-12
    assert rel(bd, d["sol_bd"]) < 1e-12
    assert st.iKs == int(d["sol_iKs"]) and st.lGMRES == int(d["sol_lGMRES"])
    assert st.ntotGM == int(d["sol_ntotGM"])
    assert abs(st.eGMRES / float(d["sol_eGMRES"]) - 1.0) < 1e-2
    if p.get("iDC", 0):
        # With discontinuity capturing itrFDI sets eGMRES = 2.4e-12 in this case (the
        # reference's ElmMFG rmes also differs from ItrRes's modified residual by e3dc.f:366,
        # rmi(:,11) = rmi(:,12) + ...), so the products (Rmod - rmes)/eGMRES amplify rounding
        # by ~1e4 and two FP64 evaluations of the same solve agree to ~2e-3 (measured, also
        # with the reference's own eGMRES); the element routines and the Krylov counts are
        # the sharp checks of this case.
        assert rel(Dy, d["sol_Dy"]) < 1e-2
    else:
        assert rel(Dy, d["sol_Dy"]) < 1e-5


@pytest.mark.parametrize("name", having("step"))
def test_oracle_time_step_matches_reference(name):
    d, case, p = load(name)
    almi, alfi, gami, Dtgl = d["setup"]
    assert (p["almi"], p["alfi"], p["gami"], p["Dtgl"]) == (almi, alfi, gami, Dtgl)
    o = pyoracle.Oracle(case, p)
    yold, acold, y, ac, stats = o.time_step(d["y"], d["ac"], 2)
    assert [s.iKs for s in stats] == list(d["step_iks"])
    assert rel(y, d["step_y"]) < 1e-9 and rel(yold, d["step_yold"]) < 1e-9
    assert rel(ac, d["step_ac"]) < 1e-7 and rel(acold, d["step_acold"]) < 1e-7


# ---- sparse solver (lhs = 1): the reference's lhsK(25, nnz_tot) is stored as a (25, nnz) array
@pytest.mark.parametrize("name", having("sparse"))
def test_oracle_genadj_matches_reference(name):
    d, case, p = load(name)
    colm, rowp = pyoracle.Oracle(case, p).genadj()
    assert np.array_equal(colm, d["sp_colm"]) and np.array_equal(rowp, d["sp_rowp"])


@pytest.mark.parametrize("name", having("sparse"))
def test_oracle_elmgmrs_matches_reference(name):
    d, case, p = load(name)
    res, bd, lhsK = pyoracle.Oracle(case, p).ElmGMRs(d["y"], d["ac"])
    assert rel(res, d["sp_res"]) < 1e-12
    assert rel(bd, d["sp_bd"]) < 1e-12
    assert rel(lhsK, d["sp_lhsK"].T) < 1e-12


@pytest.mark.parametrize("name", having("sparse"))
def test_oracle_spsi3pre_sparseap_match_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    pre = o.Spsi3pre(d["sp_lu"], d["sp_lhsK"].T)
    assert rel(pre, d["sp_pre"].T) < 1e-12
    assert rel(o.SparseAp(d["sp_pre"].T, d["sp_p"]), d["sp_ap"]) < 1e-12


@pytest.mark.parametrize("name", having("sparse"))
def test_oracle_solgmrs_matches_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    res, bd, Dy, lhsK, st = o.SolGMRs(d["y"], d["ac"])
    assert rel(res, d["sps_res"]) < 1e-12
    assert rel(bd, d["sps_bd"]) < 1e-12
    assert rel(lhsK, d["sp_pre"].T) < 1e-12
    assert (st.iKs, st.lGMRES, st.ntotGM) == (int(d["sps_iKs"]), int(d["sps_lGMRES"]), int(d["sps_ntotGM"]))
    assert rel(Dy, d["sps_Dy"]) < 1e-9


# ---- element-by-element solver: EGmass is stored as products with seeded probe vectors
def _probe(EG, v):
    return np.einsum("eij,ej->ei", EG, v)


@pytest.mark.parametrize("name", having("ebe"))
def test_oracle_elmgmre_i3pre_au1gmr_match_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    res, bd, EG = o.ElmGMRe(d["y"], d["ac"])
    assert rel(res, d["ebe_res"]) < 1e-12 and rel(bd, d["ebe_bd"]) < 1e-12
    assert rel(_probe(EG, d["ebe_v"]), d["ebe_EGv"]) < 1e-12
    pre = o.i3pre(d["ebe_lu"], EG)
    assert rel(_probe(pre, d["ebe_v"]), d["ebe_prev"]) < 1e-12
    # the golden product was formed from the reference's own preconditioned EGmass
    assert rel(o.Au1GMR(pre, d["ebe_p"]), d["ebe_ap"]) < 1e-12


@pytest.mark.parametrize("name", having("ebe"))
def test_oracle_solgmre_matches_reference(name):
    d, case, p = load(name)
    o = pyoracle.Oracle(case, p)
    res, bd, Dy, EG, st = o.SolGMRe(d["y"], d["ac"])
    assert rel(res, d["ebe_sres"]) < 1e-12 and rel(bd, d["ebe_sbd"]) < 1e-12
    assert (st.iKs, st.lGMRES, st.ntotGM) == (int(d["ebe_iKs"]), int(d["ebe_lGMRES"]), int(d["ebe_ntotGM"]))
    assert rel(Dy, d["ebe_Dy"]) < 1e-9
