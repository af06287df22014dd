"""The GMRES cycle, and the whole time step, as one CUDA graph (config no_graph = 0, the default).

Each Krylov iteration of a cycle is the body of a conditional node that the previous
iteration's Givens kernel opens while the cycle has not converged.  The graph runs the
same kernels with the same arguments in the same order as the kernel-by-kernel cycle, so
every result must be bit for bit the same: checked for the mixed-precision linearized
solver, the FP64 linearized and sparse (SolGMRs) solvers, the element-by-element solver,
restarted cycles that run to Kspace, and the finite-difference solver (which keeps the
kernel-by-kernel cycle: its product reads eGMRES as a launch value).  The mixed-precision
block-diagonal matrix-free solve with one cycle per Newton iteration runs the whole time step as
one graph (phgpu_step_graphs): the same kernels, plus two that record each Newton iteration's
statistics on the device.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import channel
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


def _steps(case, p, y, ac, no_graph, nsteps=2, nitr=2, with_steps=False):
    g = GpuSolver(case, dict(p, no_graph=no_graph))
    try:
        out = []
        for _ in range(nsteps):
            _yo, _ao, y, ac, st = g.time_step(y, ac, nitr=nitr)
            out.append((y.copy(), ac.copy(), st.iKs, g.ntotGM, st.rnorm, st.echeck))
        res = (out, g.graph_cycles, g.kernel_launches)
        return res + (g.step_graphs,) if with_steps else res
    finally:
        g.close()


@pytest.mark.parametrize("opts", [
    dict(precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR),
    dict(precision=L.PHGPU_FP64, ap_mode=L.PHGPU_AP_LINEAR),
    dict(precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, Kspace=3, nGMRES=3),
    dict(precision=L.PHGPU_FP64, ap_mode=L.PHGPU_AP_SPARSE),
    dict(precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_SPARSE, Kspace=4, nGMRES=2),
    dict(precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_EBE),
], ids=["mixed-linear", "fp64-linear", "mixed-linear-restarts", "fp64-sparse", "mixed-sparse-restarts",
        "mixed-ebe"])
def test_graph_cycle_is_bitwise_the_kernel_by_kernel_cycle(opts):
    case, p, y, ac = channel(10, ac_scale=0.05, Kspace=opts.pop("Kspace", 10), nGMRES=opts.pop("nGMRES", 1))
    p = dict(p, **opts)
    a, runs_a, la, steps_a = _steps(case, p, y, ac, no_graph=0, with_steps=True)
    b, runs_b, lb = _steps(case, p, y, ac, no_graph=1)
    assert runs_a > 0, "the cycle graph was not used"
    assert runs_b == 0
    for (ya, aa, ka, na, *_), (yb, ab, kb, nb, *_) in zip(a, b):
        assert np.array_equal(ya, yb) and np.array_equal(aa, ab)
        assert ka == kb and na == nb
    # the same kernels ran (launch counts include the graph's kernel nodes); the step graph
    # adds its two statistics kernels per Newton iteration
    assert la == lb + (2 * 2 * 2 if steps_a > 0 else 0)


def test_finite_difference_solver_keeps_the_launched_cycle():
    case, p, y, ac = channel(8, ac_scale=0.05, Kspace=10)
    p = dict(p, precision=L.PHGPU_FP64, ap_mode=L.PHGPU_AP_FD)
    _a, runs, _l = _steps(case, p, y, ac, no_graph=0, nsteps=1)
    assert runs == 0


@pytest.mark.parametrize("which", ["channel", "layered", "layered_open", "channel_idiff"])
def test_step_graph_is_bitwise_the_launched_time_step(which):
    """Whole time steps (predictor, 3 Newton iterations, update) as one graph: the state, the
    iteration counts and the statistics equal the kernel-by-kernel time steps."""
    from helpers import layered
    if which.startswith("layered"):
        case, p, y, ac = layered(6, (2, 1, 3), Kspace=20, periodic_x=which == "layered")
    else:
        case, p, y, ac = channel(10, ac_scale=0.05, Kspace=20, idiff=1 if which == "channel_idiff" else 0)
    p = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF)
    a, _ra, la, steps = _steps(case, p, y, ac, no_graph=0, nsteps=3, nitr=3, with_steps=True)
    b, _rb, lb = _steps(case, p, y, ac, no_graph=1, nsteps=3, nitr=3)
    assert steps == 3
    for (ya, aa, ka, na, ra, ea), (yb, ab, kb, nb, rb, eb) in zip(a, b):
        assert np.array_equal(ya, yb) and np.array_equal(aa, ab)
        assert ka == kb and na == nb and ra == rb and ea == eb
    assert la == lb + 2 * 3 * 3
