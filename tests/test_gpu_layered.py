"""GPU parity on one connected mesh whose element topologies share nodes.

The layered box (phasta_gb300.mesh.layered) stacks hexes, prisms and Kuhn tets in z on one
node lattice, fully periodic or open in x (inflow and outflow faces of all three topologies):
every node of a layer interface sums the contributions of two
element topologies (hex/prism, prism/tet and, through the periodic wrap, tet/hex), in the order
the GPU's colour launches give them.  Tolerances as in test_gpu_parity.py: FP64 residuals and
block diagonal 1e-10 against the oracle (and on the interface nodes alone), FP32 block diagonal
1e-5, split double-float outer residual 1e-6 of the FP64 one, FP64 time step 1e-8, assembled
tangent 1e-12 and its solve's Dy 1e-8."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import layered, rel
from oracle import pyoracle
from phasta_gb300 import _lib as L
from phasta_gb300 import mesh
from phasta_gb300.solver import GpuSolver, make_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[True, False], ids=["periodic", "open"])
def lay(request, gpu_lib):
    """The layered box, fully periodic or with a Dirichlet inflow at x = 0 and outflow at x = 1
    through boundary tets, hexes (lcsyst 2) and prisms (lcsyst 4)."""
    case, p, y, ac = layered(8, (3, 2, 3), Kspace=20, periodic_x=request.param)
    if not request.param:
        assert case.nbelem > 0 and sorted(b.lcsyst for b in case.bnd) == [2, 4]
    return case, p, y, ac, GpuSolver(case, p), pyoracle.Oracle(case, p, nthreads=4)


def _interface_nodes(case):
    """Masters touched by elements of two topologies."""
    m = lambda a: set(case.iper[np.asarray(a).reshape(-1)])  # noqa: E731
    t, h, w = m(case.ien), m(case.ienh), m(case.ienw)
    return np.array(sorted((t & h) | (t & w) | (h & w)))


def test_interfaces_exist(lay):
    case = lay[0]
    nodes = _interface_nodes(case)
    assert len(nodes) >= 3 * 8 * 8  # three interface planes of 8 x 8 masters


def test_elmmfg_fp64_and_its_interface_nodes(lay):
    case, p, y, ac, g, o = lay
    rg, mg, bg = g.ElmMFG(y, ac)
    ro, mo, bo = o.ElmMFG(y, ac)
    assert rel(rg, ro) < 1e-10 and rel(mg, mo) < 1e-10 and rel(bg, bo) < 1e-10
    n, nodes = case.nshg, _interface_nodes(case)
    idx = np.concatenate([nodes + k * n for k in range(5)])
    bidx = np.concatenate([nodes + k * n for k in range(25)])
    assert rel(rg[idx], ro[idx]) < 1e-10 and rel(mg[idx], mo[idx]) < 1e-10 and rel(bg[bidx], bo[bidx]) < 1e-10


def test_fp32_block_diagonal_and_split_residual(lay):
    case, p, y, ac, g, o = lay
    base = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR)
    _, _, bo = o.ElmMFG(y, ac)
    _, _, bm = GpuSolver(case, base).ElmMFG(y, ac)
    assert rel(bm, bo) < 1e-5
    r64, _, _, s64 = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_FP64)).SolMFG(y, ac)
    rdf, _, _, sdf = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_SPLITDF)).SolMFG(y, ac)
    assert rel(rdf, r64) < 1e-6
    assert sdf.rnorm == pytest.approx(s64.rnorm, rel=1e-7)


def test_time_step_fp64(lay):
    case, p, y, ac, g, o = lay
    yog, aog, yg, acg, _ = g.time_step(y, ac, 2)
    yoo, aoo, yo, aco, _ = o.time_step(y, ac, 2)
    assert rel(yg, yo) < 1e-8 and rel(yog, yoo) < 1e-8 and rel(aog, aoo) < 1e-5


def test_mixed_precision_newton_step(lay):
    case, p, y, ac, g, o = lay
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    gm = GpuSolver(case, dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                              outer_residual=L.PHGPU_RES_SPLITDF))
    y1, a1, st = gm.newton(y, ac, y, ac)
    yo, ao, so, _ = o.newton(y, ac, y, ac)
    assert st.echeck <= p["etol"] * st.unorm0
    assert rel(y1 - y, yo - y) < 10 * p["etol"]
    assert np.linalg.norm(o.ElmRes(y1, a1)) < np.linalg.norm(o.ElmRes(yo, ao)) + 10 * p["etol"] * r0


def test_sparse_solver(lay):
    case, p, y, ac, g, o = lay
    _, _, Dg, lg, sg = g.SolGMRs(y, ac)
    _, _, Do, lo, so = pyoracle.Oracle(case, p, nthreads=4).SolGMRs(y, ac)
    assert rel(lg, lo) < 1e-12 and rel(Dg, Do) < 1e-8 and sg.iKs == so.iKs


def test_mixed_topology_workload_at_moderate_size(gpu_lib):
    """The mixed-topology workload's layering at 32 x 32 x (16 + 2 + 12) cells with its state
    (random-phase Fourier velocity modes, k <= 8, Mach 0.35): free stream gives a zero residual,
    and a mixed-precision time step of 3 Newton iterations reduces the FP64 residual."""
    case, ph = mesh.layered_case(32, 16, 2, 12, mach=0.35)
    p = make_params(ph["mu"], ph["dt"], Kspace=20, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                    outer_residual=L.PHGPU_RES_SPLITDF)
    g = GpuSolver(case, p)
    y0 = mesh.uniform_state(case, 0.35, sigma=0.0)
    assert np.abs(g.ElmRes(y0, np.zeros_like(y0))).max() < 1e-11
    y = mesh.fourier_state(case, 0.35, kmax=8, noise=1e-3)
    ac = np.zeros_like(y)
    g.upload(y, ac, y, ac)
    r0 = g.residual_norm_dev()
    st = g.time_step_dev(3)
    assert st.echeck <= p["etol"] * st.unorm0 and st.rnorm < 0.1 * r0
