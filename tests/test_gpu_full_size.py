"""Size-independent properties at the full sizes of the benchmark definitions (GPU).

The oracle is run against the GPU at up to 16^3 x 6 elsewhere; at these sizes the
checks are properties with exact or measured answers:
  * the free stream is a steady solution: the FP64 residual of a uniform state
    vanishes to rounding (interior, hex, wedge and boundary terms alike);
  * the mixed-precision Newton iterations (FP32 assembly and Krylov vectors, the
    double-float outer residual) reach the relative nonlinear residual of the all-FP64
    iterations, and the two end states agree;
  * every linear solve meets its Krylov tolerance.
Sizes: 128^3 x 6 channel (12.6M tets, 2.15M nodes); a mixed-topology domain of an
80^3 hex block, an 80^2 x 8 wedge layer (51,200 prisms) and a 69^3 x 6 tet block
(1.97M tets); the 192^3 x 6 periodic decaying vortex (42.5M tets, 7.19M stored nodes).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel
from phasta_gb300 import _lib as L
from phasta_gb300 import mesh
from phasta_gb300.solver import GpuSolver, make_params

pytestmark = pytest.mark.gpu


def _params(ph, precision, Kspace=20):
    if precision == "mixed":
        return make_params(ph["mu"], ph["dt"], Kspace=Kspace, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                           outer_residual=L.PHGPU_RES_SPLITDF)
    return make_params(ph["mu"], ph["dt"], Kspace=Kspace)


def _newton3(case, p, y0, ac0):
    """Three Newton iterations of one time step on the resident state; (rel residual, y, stats)."""
    g = GpuSolver(case, p)
    g.upload(y0, ac0, y0, ac0)
    r0 = g.residual_norm_dev()
    stats = []
    for it in range(1, 4):
        g.set_params(iter=it)
        stats.append(g.newton_dev())
    r3 = g.residual_norm_dev()
    y, ac, _, _ = g.download()
    g.close()
    return r3 / r0, y, stats


def test_channel_128_mixed_newton_tracks_fp64(gpu_lib):
    case, ph = mesh.channel_case(128, mach=0.3, re=1000.0)
    assert case.nelem == 12_582_912 and case.nshg == 2_146_689
    g = GpuSolver(case, _params(ph, "mixed"))
    u0 = mesh.uniform_state(case, 0.3, sigma=0.0)
    assert np.abs(g.ElmRes(u0, np.zeros_like(u0))).max() < 1e-10
    g.close()
    y0 = mesh.uniform_state(case, 0.3, sigma=0.01)
    ac0 = np.zeros_like(y0)
    rm, ym, sm = _newton3(case, _params(ph, "mixed"), y0, ac0)
    rd, yd, sd = _newton3(case, _params(ph, "fp64"), y0, ac0)
    for st in sm + sd:
        assert st.echeck <= 1e-3 * st.unorm0
    assert rm < 1e-3 and rd < 1e-3
    assert abs(rm / rd - 1.0) < 0.05
    assert rel(ym, yd) < 1e-6


def test_mixed_topology_domain(gpu_lib):
    case, ph = mesh.mixed_case(69, 80, (80, 80, 4))
    assert (case.nelem, case.nhex, case.nwedge) == (1_971_054, 512_000, 51_200)
    p = _params(ph, "mixed")
    g = GpuSolver(case, p)
    u0 = mesh.uniform_state(case, 0.3, sigma=0.0)
    assert np.abs(g.ElmRes(u0, np.zeros_like(u0))).max() < 1e-10
    y0 = mesh.uniform_state(case, 0.3, sigma=0.01)
    ac0 = np.zeros_like(y0)
    r0 = np.linalg.norm(g.ElmRes(y0, ac0))
    y1, a1, st = g.newton(y0, ac0, y0, ac0)
    assert st.echeck <= 1e-3 * st.unorm0
    assert np.linalg.norm(g.ElmRes(y1, a1)) < 0.1 * r0
    g.close()
    rm, ym, _ = _newton3(case, p, y0, ac0)
    rd, yd, _ = _newton3(case, _params(ph, "fp64"), y0, ac0)
    assert rm < 1e-3 and rd < 1e-3
    assert rel(ym, yd) < 1e-6


def test_vortex_192_time_step(gpu_lib):
    case, ph = mesh.periodic_vortex_case(192)
    assert case.nelem == 42_467_328
    p = _params(ph, "mixed")
    g = GpuSolver(case, p)
    u0 = mesh.uniform_state(case, 0.1, sigma=0.0)
    assert np.abs(g.ElmRes(u0, np.zeros_like(u0))).max() < 1e-10
    g.close()
    y0 = mesh.vortex_state(case)
    ac0 = np.zeros_like(y0)
    rm, ym, sm = _newton3(case, p, y0, ac0)
    rd, yd, sd = _newton3(case, _params(ph, "fp64"), y0, ac0)
    for st in sm + sd:
        assert st.echeck <= 1e-3 * st.unorm0
    assert rm < 1e-3 and rd < 1e-3
    assert rel(ym, yd) < 1e-6
