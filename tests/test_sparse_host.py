"""CPU checks of the sparse solver's host side and of its oracle properties.

genadj (phgpu_genadj) runs on the host through the C ABI, so its colm/rowp are
checked here bit for bit against the reference's own genadj output
(tests/golden/ref_*.npz) and against the oracle's restatement on larger meshes;
its error returns mirror the reference's stops.  The oracle's assembled tangent
is checked for two size-independent properties: its diagonal blocks at nodes
without boundary conditions are the block diagonal BDiag of ElmMFG, and the
product of Spsi3pre's matrix with a vector equals L^-1 A U^-1 applied by parts.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import channel, mixed, rel, vortex
from oracle import pyoracle
from phasta_gb300 import _lib as L
from phasta_gb300.solver import PhgpuError, _MeshArrays, genadj

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from make_ref_golden import CASES  # noqa: E402

SPARSE = [(n, b) for n, b, parts in CASES if "sparse" in parts]


@pytest.mark.parametrize("name,build", SPARSE)
def test_host_genadj_matches_reference(gpu_lib, name, build):
    d = np.load(GOLDEN / f"ref_{name}.npz")
    case, p, y, ac = build()
    colm, rowp = genadj(case)
    assert np.array_equal(colm, d["sp_colm"]) and np.array_equal(rowp, d["sp_rowp"])


@pytest.mark.parametrize("build", [lambda: channel(10), lambda: vortex(9), lambda: mixed(5, 4, (4, 4, 3))])
def test_host_genadj_matches_oracle_on_larger_meshes(gpu_lib, build):
    case, p, y, ac = build()
    colm, rowp = genadj(case)
    ocolm, orowp = pyoracle.Oracle(case, p).genadj()
    assert np.array_equal(colm, ocolm) and np.array_equal(rowp, orowp)
    # rows sorted, unique, and containing the diagonal
    for i in range(case.nshg):
        r = rowp[colm[i] - 1: colm[i + 1] - 1]
        assert np.all(np.diff(r) > 0) and (i + 1) in r


def test_host_genadj_errors(gpu_lib):
    case, p, y, ac = channel(4)
    with pytest.raises(PhgpuError) as e:
        genadj(case, nnz=3)  # rows of an interior node hold 15 blocks
    assert e.value.code == L.PHGPU_ERR_TOO_LARGE
    ma = _MeshArrays(case)
    ma.ien[0] = case.nshg  # node index out of range
    colm = np.zeros(case.nshg + 1, np.int32)
    rowp = np.zeros(case.nshg * 40, np.int32)
    icnt = C.c_int()
    assert gpu_lib.phgpu_genadj(C.byref(ma.m), 40, L.iptr(colm), L.iptr(rowp), C.byref(icnt)) == L.PHGPU_ERR_INVALID


@pytest.mark.parametrize("build", [lambda: channel(8, ac_scale=0.05), lambda: mixed(4, 3, (3, 3, 2))])
def test_oracle_tangent_diagonal_is_the_block_diagonal(build):
    case, p, y, ac = build()
    o = pyoracle.Oracle(case, p)
    colm, rowp = o.genadj()
    res, bd, lhsK = o.ElmGMRs(y, ac)
    _, _, bdm = o.ElmMFG(y, ac)
    N = case.nshg
    # nodes with no boundary condition and no periodic slave (only the node itself maps to it)
    free = [i for i in range(N) if case.iBC[i] == 0 and np.sum(case.iper == i) == 1]
    assert len(free) > 0
    bdm = bdm.reshape(5, 5, N)  # bd[(r + 5 c) * N + n]
    for i in free:
        k = colm[i] - 1 + int(np.searchsorted(rowp[colm[i] - 1: colm[i + 1] - 1], i + 1))
        blk = lhsK[k].reshape(5, 5).T  # lhsK[k, 5 g + f] = (f, g)
        assert np.allclose(blk, bdm[:, :, i].T, rtol=1e-12, atol=1e-12 * np.abs(blk).max())


def test_oracle_preconditioned_product_factorizes():
    case, p, y, ac = channel(6, ac_scale=0.05)
    o = pyoracle.Oracle(case, p)
    res, bd, lhsK = o.ElmGMRs(y, ac)
    lu, _ = o.i3LU(bd, None, 0)
    pre = o.Spsi3pre(lu, lhsK)
    v = np.random.default_rng(3).standard_normal(5 * case.nshg)
    lhs = o.SparseAp(pre, v)
    # L^-1 A U^-1 v by parts: backward (U^-1), product, forward (L^-1)
    _, u = o.i3LU(lu, v, 2)
    rhs = o.SparseAp(lhsK, u)
    _, rhs = o.i3LU(lu, rhs, 1)
    assert rel(lhs, rhs) < 1e-12
