"""GPU parity: the sm_103a kernels (through the C ABI) against the CPU oracle.

Tolerances (relative, in the 2-norm over the whole array):
  * FP64 residual, modified residual, BDiag: 1e-10
  * FP64 i3LU factors and solves:            1e-12
  * FP32 block diagonal (mixed mode):        1e-5
  * finite-difference GMRES (FP64): the same Krylov iteration count, Dy within 1e-6
    (Au1MFG amplifies rounding by 1/eGMRES, so bitwise-different sums move Dy at ~1e-9)
  * mixed-precision Newton step: the nonlinear residual after the step within
    the Krylov tolerance of the FP64 step's
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import channel, mixed, rel, vortex
from oracle import pyoracle
from phasta_gb300 import _lib as L
from phasta_gb300 import mesh
from phasta_gb300.solver import GpuSolver, PhgpuError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c8(gpu_lib):
    case, p, y, ac = channel(8, ac_scale=0.05)
    return case, p, y, ac, GpuSolver(case, p), pyoracle.Oracle(case, p)


@pytest.fixture(scope="module")
def c16(gpu_lib):
    case, p, y, ac = channel(16, ac_scale=0.05)
    return case, p, y, ac, GpuSolver(case, p), pyoracle.Oracle(case, p, nthreads=4)


@pytest.mark.parametrize("which", ["c8", "c16"])
def test_elmmfg_fp64(which, request):
    case, p, y, ac, g, o = request.getfixturevalue(which)
    rg, mg, bg = g.ElmMFG(y, ac)
    ro, mo, bo = o.ElmMFG(y, ac)
    assert rel(rg, ro) < 1e-10
    assert rel(mg, mo) < 1e-10
    assert rel(bg, bo) < 1e-10


def test_elmres_and_elmmfg_without_preconditioner(c8):
    case, p, y, ac, g, o = c8
    assert rel(g.ElmRes(y, ac), o.ElmRes(y, ac)) < 1e-10
    rg, mg, _ = g.ElmMFG(y, ac, iprec=0)
    ro, mo, _ = o.ElmMFG(y, ac, iprec=0)
    assert rel(rg, ro) < 1e-10 and rel(mg, mo) < 1e-10


def test_itrres_perturbed_state(c8):
    case, p, y, ac, g, o = c8
    rng = np.random.default_rng(11)
    yp = y * (1.0 + 1e-3 * rng.standard_normal(y.shape))
    r0 = rng.standard_normal(y.shape)
    assert rel(g.ItrRes(yp, y, ac, r0), o.ItrRes(yp, y, ac, r0)) < 1e-10


def test_i3lu_all_codes(c8):
    case, p, y, ac, g, o = c8
    _, _, bd = o.ElmMFG(y, ac)
    lug, _ = g.i3LU(bd, None, L.LU_FACT)
    luo, _ = o.i3LU(bd, None, 0)
    assert rel(lug, luo) < 1e-12
    r = np.random.default_rng(3).standard_normal(5 * case.nshg)
    for code in (L.LU_FORWARD, L.LU_BACKWARD, L.LU_PRODUCT):
        _, a = g.i3LU(luo, r, code)
        _, b = o.i3LU(luo, r.copy(), code)
        assert rel(a, b) < 1e-12, code


def test_i3lu_singular_block_reports_status(c8):
    case, p, y, ac, g, o = c8
    bd = np.zeros(25 * case.nshg)
    with pytest.raises(PhgpuError) as e:
        g.i3LU(bd, None, L.LU_FACT)
    assert e.value.code == 4  # PHGPU_ERR_SINGULAR
    # the context stays usable
    assert rel(g.ElmRes(y, ac), o.ElmRes(y, ac)) < 1e-10


def test_periodic_vortex_residual(gpu_lib):
    case, p, y, ac = vortex(8)
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    rg, mg, bg = g.ElmMFG(y, ac)
    ro, mo, bo = o.ElmMFG(y, ac)
    assert rel(rg, ro) < 1e-10 and rel(mg, mo) < 1e-10 and rel(bg, bo) < 1e-10


def test_solmfg_fd_matches_oracle(c8):
    case, p, y, ac, g, o = c8
    rg, bg, Dg, sg = g.SolMFG(y, ac)
    ro, bo, Do, so = o.SolMFG(y, ac)
    assert rel(rg, ro) < 1e-10
    assert rel(bg, bo) < 1e-10
    # itrFDI differences residuals at sqrt(epsM): rounding differences of the
    # two implementations reach ~1e-5 of the interval
    assert abs(sg.eGMRES - so.eGMRES) <= 1e-3 * so.eGMRES
    assert sg.iKs == so.iKs
    assert rel(Dg, Do) < 1e-6
    assert sg.echeck <= p["etol"] * sg.unorm0


def test_newton_step_fp64_matches_oracle(c16):
    case, p, y, ac, g, o = c16
    yg, acg, sg = g.newton(y, ac, y, ac)
    yo, aco, so, _ = o.newton(y, ac, y, ac)
    assert rel(yg, yo) < 1e-9
    assert rel(acg, aco) < 1e-6
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    assert np.linalg.norm(o.ElmRes(yg, acg)) < 0.05 * r0


def test_linearized_product_agrees_with_finite_difference(gpu_lib):
    """The linearized Jacobian-vector product is the eps -> 0 limit of Au1MFG."""
    case, p, y, ac = channel(8)
    p_lin = dict(p, ap_mode=L.PHGPU_AP_LINEAR)
    g_fd, g_lin = GpuSolver(case, p), GpuSolver(case, p_lin)
    _, _, Dfd, sfd = g_fd.SolMFG(y, ac)
    _, _, Dlin, slin = g_lin.SolMFG(y, ac)
    assert abs(sfd.iKs - slin.iKs) <= 1
    # both solve J Dy = R to the Krylov tolerance; they differ by O(eGMRES) and the tolerance
    assert rel(Dlin, Dfd) < 5 * p["etol"]


def test_mixed_precision_newton_step(gpu_lib):
    case, p, y, ac = channel(16)
    p64 = dict(p, ap_mode=L.PHGPU_AP_LINEAR)
    pmx = dict(p, ap_mode=L.PHGPU_AP_LINEAR, precision=L.PHGPU_MIXED)
    o = pyoracle.Oracle(case, p, nthreads=4)
    g64, gmx = GpuSolver(case, p64), GpuSolver(case, pmx)
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    y64, a64, s64 = g64.newton(y, ac, y, ac)
    ymx, amx, smx = gmx.newton(y, ac, y, ac)
    r64 = np.linalg.norm(o.ElmRes(y64, a64))
    rmx = np.linalg.norm(o.ElmRes(ymx, amx))
    assert abs(smx.iKs - s64.iKs) <= 2
    # the correction agrees to the Krylov tolerance, so do the new residuals
    assert rel(ymx - y, y64 - y) < 10 * p["etol"]
    assert rmx < r64 + 10 * p["etol"] * r0
    assert s64.rnorm == pytest.approx(r0, rel=1e-10)
    assert smx.rnorm == pytest.approx(r0, rel=1e-10)  # the outer residual is FP64 in both modes


def test_time_step_matches_oracle(gpu_lib):
    case, p, y, ac = channel(8)
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    yog, aog, yg, acg, sg = g.time_step(y, ac, 2)
    yoo, aoo, yo, aco, so = o.time_step(y, ac, 2)
    assert rel(yg, yo) < 1e-8
    assert rel(yog, yoo) < 1e-8
    assert rel(aog, aoo) < 1e-5


def test_nan_state_reports_nonfinite_and_context_survives(c8):
    case, p, y, ac, g, o = c8
    bad = y.copy()
    bad[5] = np.nan
    with pytest.raises(PhgpuError) as e:
        g.SolMFG(bad, ac)
    assert e.value.code in (3, 4)
    assert rel(g.ElmRes(y, ac), o.ElmRes(y, ac)) < 1e-10


def test_deterministic_repeat(c16):
    case, p, y, ac, g, o = c16
    a = g.ElmMFG(y, ac)
    b = g.ElmMFG(y, ac)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("n", [48])
def test_large_mesh_properties(gpu_lib, n):
    """Size-independent properties at a mesh the oracle is not run on."""
    case, ph = mesh.channel_case(n)
    from phasta_gb300.solver import make_params
    p = make_params(ph["mu"], ph["dt"], Kspace=20, ap_mode=L.PHGPU_AP_LINEAR, precision=L.PHGPU_MIXED)
    g = GpuSolver(case, p)
    y0 = mesh.uniform_state(case, 0.3, sigma=0.0)
    ac = np.zeros_like(y0)
    r = g.ElmRes(y0, ac)
    assert np.abs(r).max() < 1e-11  # free stream
    y = mesh.uniform_state(case, 0.3)
    r0 = np.linalg.norm(g.ElmRes(y, ac))
    y1, a1, st = g.newton(y, ac, y, ac)
    assert st.echeck <= p["etol"] * st.unorm0
    assert np.linalg.norm(g.ElmRes(y1, a1)) < 0.1 * r0


def test_galerkin64_outer_residual_against_fp64(gpu_lib):
    """Mixed-precision outer residual (FP64 Galerkin terms, FP32 stabilization) vs all-FP64."""
    case, p, y, ac = channel(16, ac_scale=0.05)
    pm = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_GALERKIN64)
    g = GpuSolver(case, pm)
    o = pyoracle.Oracle(case, p, nthreads=4)
    _, _, _, st = g.SolMFG(y, ac)
    r64 = np.linalg.norm(o.ElmRes(y, ac))
    # the residual norm the solver used agrees with the all-FP64 residual to FP32 rounding of
    # the stabilization and viscous terms
    assert st.rnorm == pytest.approx(r64, rel=1e-5)
    y1, a1, st1 = g.newton(y, ac, y, ac)
    assert np.linalg.norm(o.ElmRes(y1, a1)) < 0.05 * r64


@pytest.mark.parametrize("which", ["channel", "vortex", "channel_idiff"])
def test_split_double_float_outer_residual(gpu_lib, which):
    """Outer residual with no FP64 arithmetic (double-float element-constant Euler flux, FP32
    increments and stabilization) against the FP64 outer residual of the same mixed solve.

    The runs share the FP32 block diagonal, so res = L^-1 R differs only through R.  The
    gradients come from double-float node differences, so the FP32 stabilization, viscous
    and time terms carry FP32 accuracy relative to their own size, as does the flux
    increment over an element.  Tolerances: 1e-6 relative on the channel (observed 2e-7);
    1e-5 on the 8^3 vortex (observed 4e-6), whose elements span 2 pi / 8, so the increments
    are as large as the flux itself; in both cases at least 3x closer to FP64 than the
    FP64-Galerkin hybrid, whose FP32 gradients of rounded nodal values are less accurate."""
    if which == "vortex":
        case, p, y, ac = vortex(8)
    else:
        case, p, y, ac = channel(16, ac_scale=0.05, idiff=1 if which == "channel_idiff" else 0)
    base = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR)
    r64, _, _, s64 = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_FP64)).SolMFG(y, ac)
    rdf, _, _, sdf = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_SPLITDF)).SolMFG(y, ac)
    assert rel(rdf, r64) < (1e-5 if which == "vortex" else 1e-6)
    assert sdf.rnorm == pytest.approx(s64.rnorm, rel=1e-7)
    if which != "channel_idiff":  # the FP64-Galerkin hybrid does not take idiff = 1
        rgl, _, _, sgl = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_GALERKIN64)).SolMFG(y, ac)
        assert rel(rdf, r64) < rel(rgl, r64) / 3


@pytest.mark.parametrize("idiff", [0, 1])
def test_split_double_float_outer_residual_hex_wedge(gpu_lib, idiff):
    """The split residual of the hex and wedge blocks (element-constant flux through the
    FP64-formed integrals I_a,i = sum_q W_q N_a,i in double-float, FP32 increments) against
    the FP64 outer residual of the same mixed solve, on disjoint tet/hex/wedge blocks with the
    channel's perturbed free stream.  Tolerance 1e-6 relative, as for the tet channel."""
    case, p, y, ac = mixed(6, 6, (6, 6, 3), idiff=idiff)
    base = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR)
    r64, _, _, s64 = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_FP64)).SolMFG(y, ac)
    rdf, _, _, sdf = GpuSolver(case, dict(base, outer_residual=L.PHGPU_RES_SPLITDF)).SolMFG(y, ac)
    assert rel(rdf, r64) < 1e-6
    assert sdf.rnorm == pytest.approx(s64.rnorm, rel=1e-7)



@pytest.mark.parametrize("which", ["hex", "wedge"])
def test_mixed_newton_on_tet_free_meshes(gpu_lib, which):
    """Meshes with no tets (the channel on hexes, the channel on prisms with triangle walls): the
    FP32 products of the hexes and prisms read the packed node records that every write of the
    FP32 state refreshes.  A mixed-precision Newton step against the oracle's FP64 one: the
    update within 10 x the Krylov tolerance, the residual no larger than the oracle's plus that."""
    from helpers import hexchannel, wedgechannel
    case, p, y, ac = hexchannel(6) if which == "hex" else wedgechannel((6, 6, 4))
    p = dict(p, Kspace=20)
    o = pyoracle.Oracle(case, p)
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    gm = GpuSolver(case, dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                              outer_residual=L.PHGPU_RES_SPLITDF))
    y1, a1, st = gm.newton(y, ac, y, ac)
    yo, ao, so, _ = o.newton(y, ac, y, ac)
    assert st.echeck <= p["etol"] * st.unorm0
    assert rel(y1 - y, yo - y) < 10 * p["etol"]
    assert np.linalg.norm(o.ElmRes(y1, a1)) < np.linalg.norm(o.ElmRes(yo, ao)) + 10 * p["etol"] * r0


@pytest.mark.parametrize("iDC", [1, 2, 3])
@pytest.mark.parametrize("make", [lambda iDC: channel(10, ac_scale=0.05, sigma=0.05, iDC=iDC),
                                  lambda iDC: mixed(3, 3, (3, 3, 2), sigma=0.05, iDC=iDC)],
                         ids=["channel10", "mixed3"])
def test_discontinuity_capturing_fp64(gpu_lib, make, iDC):
    """iDC = 1, 2, 3 (e3dc.f) in the FP64 element routines: ElmMFG's res, rmes (with the
    reference's rmi(:,11) line) and BDiag, ItrRes's modified residual, within 1e-10 of the
    oracle; the DC term itself is non-trivial (the residual moves against iDC = 0)."""
    case, p, y, ac = make(iDC)
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    r, m, b = g.ElmMFG(y, ac)
    ro, mo, bo = o.ElmMFG(y, ac)
    assert rel(r, ro) < 1e-10 and rel(m, mo) < 1e-10 and rel(b, bo) < 1e-10
    g0 = GpuSolver(case, dict(p, iDC=0))
    r0, m0, _b0 = g0.ElmMFG(y, ac)
    assert rel(r, r0) > 1e-6 and rel(m, m0) > 1e-6
    rng = np.random.default_rng(5)
    yp = y * (1.0 + 1e-3 * rng.standard_normal(y.shape))
    base = rng.standard_normal(y.shape)
    assert rel(g.ItrRes(yp, y, ac, base), o.ItrRes(yp, y, ac, base)) < 1e-10
    g.close()
    g0.close()


def test_discontinuity_capturing_needs_fp64_fd(gpu_lib):
    case, p, y, ac = channel(6, iDC=1, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR)
    g = GpuSolver(case, p)
    with pytest.raises(PhgpuError) as e:
        g.SolMFG(y, ac)
    assert e.value.code == L.PHGPU_ERR_UNSUPPORTED


@pytest.mark.parametrize("make", [lambda: channel(10, ac_scale=0.05, itau=1),
                                  lambda: mixed(3, 3, (3, 3, 2), itau=1)], ids=["channel10", "mixed3"])
def test_franca_tau_fp64(gpu_lib, make):
    """itau = 1 (Diagonal-Franca tau, e3tau.f:54-139) in the FP64 kernels: ElmMFG, ItrRes and
    the assembled tangent within 1e-10 / 1e-12 of the oracle, and a SolMFG with the same Krylov
    count; the tau differs from itau = 0 (the residual moves)."""
    case, p, y, ac = make()
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    r, m, b = g.ElmMFG(y, ac)
    ro, mo, bo = o.ElmMFG(y, ac)
    assert rel(r, ro) < 1e-10 and rel(m, mo) < 1e-10 and rel(b, bo) < 1e-10
    r0, _m0, _b0 = GpuSolver(case, dict(p, itau=0)).ElmMFG(y, ac)
    assert rel(r, r0) > 1e-6
    rng = np.random.default_rng(5)
    yp = y * (1.0 + 1e-3 * rng.standard_normal(y.shape))
    base = rng.standard_normal(y.shape)
    assert rel(g.ItrRes(yp, y, ac, base), o.ItrRes(yp, y, ac, base)) < 1e-10
    res, bd, Dy, st = g.SolMFG(y, ac)
    ores, obd, oDy, ost = o.SolMFG(y, ac)
    assert st.iKs == ost.iKs and rel(Dy, oDy) < 1e-6
    _gres, _gbd, lhsK = g.ElmGMRs(y, ac)
    _ores, _obd, olhsK = o.ElmGMRs(y, ac)
    assert rel(lhsK, olhsK) < 1e-12


@pytest.mark.parametrize("n,idiff", [(10, 0), (64, 0), (12, 1)])
def test_pipelined_linearized_product_is_the_per_chunk_kernel(gpu_lib, n, idiff):
    """The persistent cp.async-pipelined FP32 linearized product and split outer residual
    (config no_pipe = 0) against one CTA per chunk (no_pipe = 1): the same arithmetic and
    summation order, so a mixed-precision time step is bitwise the same.  At 64^3 x 6 the
    colours hold more chunks than the persistent grid, so CTAs walk several chunks through
    both halves of the buffers; idiff = 1 stages the reconstructed flux as well."""
    case, p, y, ac = channel(n, ac_scale=0.05, Kspace=6, idiff=idiff)
    p = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF)
    out = []
    for no_pipe in (0, 1):
        g = GpuSolver(case, dict(p, no_pipe=no_pipe))
        # the pipelined variants compiled for the per-chunk kernels' occupancy (4 and 3 CTAs/SM)
        g.set_tuning(4, 3)
        _yo, _ao, y1, a1, st = g.time_step(y, ac, nitr=1)
        out.append((y1, a1, st.iKs))
        g.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_time_step_on_pinned_host_buffers(gpu_lib):
    """The host-buffer time step on page-locked arrays (the e2e path of the bench) is bitwise
    the one on pageable arrays."""
    torch = pytest.importorskip("torch")
    case, p, y, ac = channel(8, ac_scale=0.05, Kspace=10)
    g = GpuSolver(case, p)
    yo1, ao1, y1, a1, _st = g.time_step(y, ac, nitr=2)
    g.close()

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = a.reshape(-1)
        return t, t.numpy()

    keep = [pinned(y), pinned(ac), pinned(np.zeros_like(y)), pinned(np.zeros_like(ac))]
    yo, ao, y2, a2 = (k[1] for k in keep)
    g2 = GpuSolver(case, p)
    g2.time_step_into(yo, ao, y2, a2, nitr=2)
    g2.close()
    assert np.array_equal(y2, y1.reshape(-1)) and np.array_equal(a2, a1.reshape(-1))
    assert np.array_equal(yo, yo1.reshape(-1)) and np.array_equal(ao, ao1.reshape(-1))
