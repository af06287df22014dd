"""GPU parity of the element-by-element solver (the reference's impl = 3x path).

Against the reference's own outputs (tests/golden/ref_*.npz, "ebe" part): ElmGMRe
(res, BDiag, and the element tangents EGmass through products with seeded probe
vectors), i3pre, Au1GMR with bc3per, and SolGMRe; against the oracle on larger
single-topology meshes.  Tolerances (relative 2-norm) as for the sparse solver:
res/BDiag 1e-10, EGmass probes and products 1e-12, SolGMRe Dy 1e-8 with the same
iteration and cycle counts; the FP32 solve tracks the FP64 one within 1e-4.  A mesh
with more than one element topology is refused (the reference's i3pre is only
correct on single-topology meshes).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import channel, mixed, rel, vortex
from oracle import pyoracle
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver, PhgpuError

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from make_ref_golden import CASES  # noqa: E402

pytestmark = pytest.mark.gpu
EBE = [(n, b) for n, b, parts in CASES if "ebe" in parts]
LARGER = [("channel10", lambda: channel(10, ac_scale=0.05)), ("vortex8", lambda: vortex(8)),
          ("hex6", lambda: mixed(0, 6, 0)), ("wedge6", lambda: mixed(0, 0, (6, 6, 4)))]


def _probe(EG, v):
    return np.einsum("eij,ej->ei", EG, v)


def load(name, build):
    d = dict(np.load(GOLDEN / f"ref_{name}.npz", allow_pickle=False))
    case, p, y, ac = build()
    assert np.array_equal(d["y"], y) and np.array_equal(d["ac"], ac)
    return d, case, p


@pytest.mark.parametrize("name,build", EBE)
def test_gpu_elmgmre_i3pre_au1gmr_match_reference(gpu_lib, name, build):
    d, case, p = load(name, build)
    g = GpuSolver(case, p)
    res, bd, EG = g.ElmGMRe(d["y"], d["ac"])
    assert rel(res, d["ebe_res"]) < 1e-10 and rel(bd, d["ebe_bd"]) < 1e-10
    assert rel(_probe(EG, d["ebe_v"]), d["ebe_EGv"]) < 1e-12
    pre = g.i3pre(d["ebe_lu"], EG)
    assert rel(_probe(pre, d["ebe_v"]), d["ebe_prev"]) < 1e-12
    assert rel(g.Au1GMR(pre, d["ebe_p"]), d["ebe_ap"]) < 1e-12


@pytest.mark.parametrize("name,build", EBE)
def test_gpu_solgmre_matches_reference(gpu_lib, name, build):
    d, case, p = load(name, build)
    g = GpuSolver(case, p)
    res, bd, Dy, EG, st = g.SolGMRe(d["y"], d["ac"])
    assert (st.iKs, st.lGMRES, st.ntotGM) == (int(d["ebe_iKs"]), int(d["ebe_lGMRES"]), int(d["ebe_ntotGM"]))
    assert rel(res, d["ebe_sres"]) < 1e-10 and rel(bd, d["ebe_sbd"]) < 1e-10
    assert rel(Dy, d["ebe_Dy"]) < 1e-8


@pytest.mark.parametrize("name,build", LARGER)
def test_gpu_ebe_matches_oracle(gpu_lib, name, build):
    case, p, y, ac = build()
    g = GpuSolver(case, p)
    o = pyoracle.Oracle(case, p, nthreads=8)
    res, bd, EG = g.ElmGMRe(y, ac)
    ores, obd, oEG = o.ElmGMRe(y, ac)
    assert rel(res, ores) < 1e-10 and rel(bd, obd) < 1e-10
    assert rel(EG, oEG) < 1e-12
    _, _, Dy, _, st = g.SolGMRe(y, ac)
    _, _, oDy, _, ost = pyoracle.Oracle(case, p, nthreads=8).SolGMRe(y, ac)
    assert (st.iKs, st.lGMRES) == (ost.iKs, ost.lGMRES)
    assert rel(Dy, oDy) < 1e-8


def test_gpu_ebe_refuses_mixed_topology(gpu_lib):
    case, p, y, ac = mixed(3, 3, (3, 3, 2))
    g = GpuSolver(case, p)
    with pytest.raises(PhgpuError) as e:
        g.SolGMRe(y, ac)
    assert e.value.code == L.PHGPU_ERR_UNSUPPORTED


@pytest.mark.parametrize("build", [lambda: channel(12, ac_scale=0.05), lambda: mixed(0, 6, 0)])
def test_gpu_mixed_ebe_solve_tracks_fp64(gpu_lib, build):
    case, p, y, ac = build()
    _, _, Dy64, _, st64 = GpuSolver(case, p).SolGMRe(y, ac)
    pm = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_EBE, outer_residual=L.PHGPU_RES_FP64)
    _, _, Dy32, eg, st32 = GpuSolver(case, pm).SolGMRe(y, ac)
    assert eg is None
    assert abs(st32.iKs - st64.iKs) <= 1
    assert rel(Dy32, Dy64) < 1e-4


def test_gpu_newton_with_the_ebe_solver_matches_oracle(gpu_lib):
    case, p, y, ac = channel(8, ac_scale=0.05)
    p = dict(p, ap_mode=L.PHGPU_AP_EBE)
    g = GpuSolver(case, p)
    y1, ac1, st = g.newton(y, ac, y, ac)
    o = pyoracle.Oracle(case, p)
    _, _, oDy, _, ost = o.SolGMRe(y, ac)
    oy, oac = o.itrCorrect(y, ac, y, ac, oDy)
    assert st.iKs == ost.iKs
    assert rel(y1, oy) < 1e-12 and rel(ac1, oac) < 1e-9
