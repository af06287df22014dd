"""GPU parity of the sparse solver (the reference's impl = 1x path, lhs = 1).

Against the reference's own outputs (tests/golden/ref_*.npz, "sparse" part):
genadj/ElmGMRs (res, BDiag, assembled tangent lhsK), Spsi3pre, SparseAp with
bc3per, and SolGMRs.  Against the oracle on larger meshes: the tangent and the
SolGMRs solution.  Tolerances (relative 2-norm): FP64 res/BDiag 1e-10 (as
ElmMFG), lhsK and the preconditioned lhsK 1e-12 (the tangent sums the same
terms in another order), SparseAp 1e-12, SolGMRs Dy 1e-8 with the same Krylov
iteration and cycle counts (GMRES on the assembled matrix is deterministic; the
bound covers rounding amplified by the Arnoldi process).  The mixed-precision
solve (FP32 tangent, FP32 Krylov vectors) is compared with the FP64 one:
Dy within 1e-4.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import channel, mixed, rel, vortex
from oracle import pyoracle
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from make_ref_golden import CASES  # noqa: E402

pytestmark = pytest.mark.gpu
SPARSE = [(n, b) for n, b, parts in CASES if "sparse" in parts]
LARGER = [("channel12", lambda: channel(12, ac_scale=0.05)), ("vortex10", lambda: vortex(10)),
          ("mixed6", lambda: mixed(6, 5, (5, 5, 4)))]


def load(name, build):
    d = dict(np.load(GOLDEN / f"ref_{name}.npz", allow_pickle=False))
    case, p, y, ac = build()
    assert np.array_equal(d["y"], y) and np.array_equal(d["ac"], ac)
    return d, case, p


@pytest.mark.parametrize("name,build", SPARSE)
def test_gpu_elmgmrs_matches_reference(gpu_lib, name, build):
    d, case, p = load(name, build)
    g = GpuSolver(case, p)
    assert g.nnz_tot == len(d["sp_rowp"])
    res, bd, lhsK = g.ElmGMRs(d["y"], d["ac"])
    assert rel(res, d["sp_res"]) < 1e-10
    assert rel(bd, d["sp_bd"]) < 1e-10
    assert rel(lhsK, d["sp_lhsK"].T) < 1e-12


@pytest.mark.parametrize("name,build", SPARSE)
def test_gpu_spsi3pre_sparseap_match_reference(gpu_lib, name, build):
    d, case, p = load(name, build)
    g = GpuSolver(case, p)
    assert rel(g.Spsi3pre(d["sp_lu"], d["sp_lhsK"].T), d["sp_pre"].T) < 1e-12
    assert rel(g.SparseAp(d["sp_pre"].T, d["sp_p"]), d["sp_ap"]) < 1e-12


@pytest.mark.parametrize("name,build", SPARSE)
def test_gpu_solgmrs_matches_reference(gpu_lib, name, build):
    d, case, p = load(name, build)
    g = GpuSolver(case, p)
    res, bd, Dy, lhsK, st = g.SolGMRs(d["y"], d["ac"])
    assert (st.iKs, st.lGMRES, st.ntotGM) == (int(d["sps_iKs"]), int(d["sps_lGMRES"]), int(d["sps_ntotGM"]))
    assert rel(res, d["sps_res"]) < 1e-10
    assert rel(bd, d["sps_bd"]) < 1e-10
    assert rel(lhsK, d["sp_pre"].T) < 1e-12
    assert rel(Dy, d["sps_Dy"]) < 1e-8


@pytest.mark.parametrize("name,build", LARGER)
def test_gpu_tangent_and_solgmrs_match_oracle(gpu_lib, name, build):
    case, p, y, ac = build()
    g = GpuSolver(case, p)
    o = pyoracle.Oracle(case, p, nthreads=8)
    res, bd, lhsK = g.ElmGMRs(y, ac)
    ores, obd, olhsK = o.ElmGMRs(y, ac)
    assert rel(res, ores) < 1e-10 and rel(bd, obd) < 1e-10
    assert rel(lhsK, olhsK) < 1e-12
    _, _, Dy, _, st = g.SolGMRs(y, ac)
    o2 = pyoracle.Oracle(case, p, nthreads=8)
    _, _, oDy, _, ost = o2.SolGMRs(y, ac)
    assert (st.iKs, st.lGMRES) == (ost.iKs, ost.lGMRES)
    assert rel(Dy, oDy) < 1e-8


def test_gpu_solgmrs_reuses_the_tangent(gpu_lib):
    case, p, y, ac = channel(8, ac_scale=0.05)
    g = GpuSolver(case, p)
    with pytest.raises(Exception):
        g.SolGMRs(y, ac, lhs=0)  # nothing assembled yet
    _, _, Dy1, lhsK1, st1 = g.SolGMRs(y, ac, lhs=1)
    _, _, Dy0, lhsK0, st0 = g.SolGMRs(y, ac, lhs=0)
    assert st0.iKs == st1.iKs
    assert np.array_equal(lhsK0, lhsK1)
    # lhs = 0 forms the residual with the residual-only kernel (lhs = 1 with the kernel that
    # also forms BDiag), so Dy agrees to rounding, not bit for bit
    assert rel(Dy0, Dy1) < 1e-12


@pytest.mark.parametrize("build", [lambda: channel(12, ac_scale=0.05), lambda: mixed(6, 5, (5, 5, 4))])
def test_gpu_mixed_sparse_solve_tracks_fp64(gpu_lib, build):
    case, p, y, ac = build()
    g64 = GpuSolver(case, dict(p, ap_mode=L.PHGPU_AP_SPARSE))
    _, _, Dy64, _, st64 = g64.SolGMRs(y, ac)
    pm = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_SPARSE, outer_residual=L.PHGPU_RES_FP64)
    g32 = GpuSolver(case, pm)
    _, _, Dy32, lk, st32 = g32.SolGMRs(y, ac)
    assert lk is None
    assert abs(st32.iKs - st64.iKs) <= 1
    assert rel(Dy32, Dy64) < 1e-4


def test_gpu_newton_with_the_sparse_solver_matches_oracle(gpu_lib):
    case, p, y, ac = channel(8, ac_scale=0.05)
    p = dict(p, ap_mode=L.PHGPU_AP_SPARSE)
    g = GpuSolver(case, p)
    y1, ac1, st = g.newton(y, ac, y, ac)
    o = pyoracle.Oracle(case, p)
    _, _, oDy, _, ost = o.SolGMRs(y, ac)
    oy, oac = o.itrCorrect(y, ac, y, ac, oDy)
    assert st.iKs == ost.iKs
    assert rel(y1, oy) < 1e-12 and rel(ac1, oac) < 1e-9
