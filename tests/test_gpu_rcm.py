"""The CUDA path on a reverse Cuthill-McKee renumbered mesh: every result is the renumbered
result of the original mesh (node order changes only the order of the floating-point sums)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import channel, layered, rel
from phasta_gb300 import _lib as L
from phasta_gb300 import mesh
from phasta_gb300.solver import GpuSolver, rcm_order

pytestmark = pytest.mark.gpu


def _shuffled_and_rcm(case):
    shuf = np.random.default_rng(11).permutation(case.nshg)
    a = mesh.renumber(case, shuf)
    p, _, _ = rcm_order(a)
    return a, p, mesh.renumber(a, p)


@pytest.mark.parametrize("which", ["channel", "layered"])
def test_fp64_elmmfg_is_equivariant_under_rcm(which):
    case, p, y, ac = channel(8, ac_scale=0.05) if which == "channel" else layered(5, (2, 1, 3))
    p = dict(p, precision=L.PHGPU_FP64)
    a, perm, b = _shuffled_and_rcm(case)
    # the state in a's numbering, then in b's
    shuf = np.random.default_rng(11).permutation(case.nshg)
    ya, aca = mesh.renumber_field(y, shuf, 5), mesh.renumber_field(ac, shuf, 5)
    yb, acb = mesh.renumber_field(ya, perm, 5), mesh.renumber_field(aca, perm, 5)
    ga, gb = GpuSolver(a, p), GpuSolver(b, p)
    try:
        ra = ga.ElmMFG(ya, aca)
        rb = gb.ElmMFG(yb, acb)
    finally:
        ga.close()
        gb.close()
    for va, vb, nc in zip(ra, rb, (5, 5, 25)):
        assert rel(mesh.renumber_field(va, perm, nc), vb) <= 1e-12


def test_mixed_time_step_on_rcm_mesh_reaches_the_same_state():
    case, p, y, ac = channel(10, ac_scale=0.05, Kspace=20)
    p = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF)
    a, perm, b = _shuffled_and_rcm(case)
    shuf = np.random.default_rng(11).permutation(case.nshg)
    ya, aca = mesh.renumber_field(y, shuf, 5), mesh.renumber_field(ac, shuf, 5)
    yb, acb = mesh.renumber_field(ya, perm, 5), mesh.renumber_field(aca, perm, 5)
    out = []
    for m, yy, aa in ((a, ya, aca), (b, yb, acb)):
        g = GpuSolver(m, p)
        try:
            _yo, _ao, y1, ac1, st = g.time_step(yy, aa, nitr=3)
            out.append((y1, st))
        finally:
            g.close()
    (y_a, st_a), (y_b, st_b) = out
    # both are three Newton iterations with Krylov tolerance 1e-3 towards the same solution; the
    # FP32 sums in another order change the iterates at the level of the nonlinear residual left
    assert rel(mesh.renumber_field(y_a, perm, 5), y_b) <= 1e-5
    assert 0.5 <= st_a.rnorm / st_b.rnorm <= 2.0
