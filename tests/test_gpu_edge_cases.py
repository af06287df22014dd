"""Edge cases on the GPU: meshes smaller than one chunk, and the checks of phgpu_create that
run after the device is set up.

* A chunk holds 128 tets (16 hexes, 21 prisms per CTA of the hex and prism kernels); the
  meshes here have 48 tets, 8 hexes, 16 prisms: one ragged chunk or CTA, colours with a
  single element, persistent grids larger than their colours.  FP64 element routines within
  1e-10 of the oracle, the mixed-precision Newton step within the Krylov tolerance of the
  oracle's FP64 one.
* Boundary hex and wedge blocks are checked when the context uploads them: a topology other
  than lcsyst 2, 3, 4 or connectivity outside the nodes is PHGPU_ERR_INVALID, and the failed
  create leaves no context behind.
* The bounded mbarrier wait that guards the pipelined sweeps' bulk copies, made to run out on a
  phase that can never complete: it gives up and reports the sweeps' copy-failure value, and
  the device stays usable.
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np
import pytest

from helpers import channel, hexchannel, mixed, rel, vortex, wedgechannel
from oracle import pyoracle
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver, PhgpuError

pytestmark = pytest.mark.gpu

TINY = [
    ("channel2", lambda: channel(2, ac_scale=0.05)),
    ("vortex2", lambda: vortex(2)),
    ("hexchannel2", lambda: hexchannel(2)),
    ("wedgechannel2", lambda: wedgechannel((2, 2, 2))),
    ("mixed2", lambda: mixed(2, 2, (2, 2, 1))),
]


@pytest.mark.parametrize("name,make", TINY, ids=[t[0] for t in TINY])
def test_meshes_smaller_than_a_chunk_fp64(gpu_lib, name, make):
    case, p, y, ac = make()
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    try:
        r, m, b = g.ElmMFG(y, ac)
        ro, mo, bo = o.ElmMFG(y, ac)
        assert rel(r, ro) < 1e-10 and rel(m, mo) < 1e-10 and rel(b, bo) < 1e-10
        rng = np.random.default_rng(7)
        yp = y * (1.0 + 1e-3 * rng.standard_normal(y.shape))
        base = rng.standard_normal(y.shape)
        assert rel(g.ItrRes(yp, y, ac, base), o.ItrRes(yp, y, ac, base)) < 1e-10
    finally:
        g.close()


@pytest.mark.parametrize("name,make", TINY, ids=[t[0] for t in TINY])
def test_meshes_smaller_than_a_chunk_mixed_newton(gpu_lib, name, make):
    case, p, y, ac = make()
    p = dict(p, Kspace=20)
    o = pyoracle.Oracle(case, p)
    r0 = np.linalg.norm(o.ElmRes(y, ac))
    g = GpuSolver(case, dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                             outer_residual=L.PHGPU_RES_SPLITDF))
    try:
        y1, a1, st = g.newton(y, ac, y, ac)
    finally:
        g.close()
    yo, ao, _so, _ = o.newton(y, ac, y, ac)
    assert st.echeck <= p["etol"] * st.unorm0
    assert rel(y1 - y, yo - y) < 10 * p["etol"]
    assert np.linalg.norm(o.ElmRes(y1, a1)) < np.linalg.norm(o.ElmRes(yo, ao)) + 10 * p["etol"] * r0


@pytest.mark.parametrize("which", ["hex", "wedge"])
def test_boundary_blocks_are_checked(gpu_lib, which):
    case, p, y, ac = hexchannel(2) if which == "hex" else wedgechannel((2, 2, 2))
    assert case.bnd, "the channel on hexes and prisms has boundary blocks"
    GpuSolver(case, p).close()  # the unmodified mesh is accepted

    bad_topology = copy.deepcopy(case)
    bad_topology.bnd[0].lcsyst = 5
    with pytest.raises(PhgpuError) as e:
        GpuSolver(bad_topology, p)
    assert e.value.code == L.PHGPU_ERR_INVALID

    bad_node = copy.deepcopy(case)
    bad_node.bnd[-1].ien[0, 1] = case.nshg
    with pytest.raises(PhgpuError) as e:
        GpuSolver(bad_node, p)
    assert e.value.code == L.PHGPU_ERR_INVALID

    # the context still works after the failed creates
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    try:
        assert rel(g.ElmRes(y, ac), o.ElmRes(y, ac)) < 1e-10
    finally:
        g.close()


def test_bounded_wait_runs_out_and_reports(gpu_lib):
    """phgpu_selftest_wait_limit: one CTA arms an mbarrier for two arrivals, gives it one and
    waits through mbar_wait, the wait of every bulk copy of the pipelined sweeps, with a small
    try limit: the wait gives up and the status is 8, the value a sweep writes to its error word
    before its CTA ends (the solve then returns PHGPU_ERR_CUDA)."""
    import time
    per_try = []
    for tries in (1, 64, 1024):
        st = C.c_int(-1)
        t0 = time.perf_counter()
        assert gpu_lib.phgpu_selftest_wait_limit(tries, C.byref(st)) == 0
        dt = time.perf_counter() - t0
        assert st.value == 8
        per_try.append(dt / tries)
    # each try suspends the thread for at most a hardware-chosen time: the sweeps' 2^19 tries
    # must end within seconds
    print(f"bounded wait: {1e6 * per_try[-1]:.2f} us per try, 2^19 tries ~ {per_try[-1] * 524288:.1f} s")
    assert per_try[-1] * 524288 < 10.0
    # the device and the library are usable afterwards
    case, p, y, ac = channel(4)
    g, o = GpuSolver(case, p), pyoracle.Oracle(case, p)
    try:
        assert rel(g.ElmRes(y, ac), o.ElmRes(y, ac)) < 1e-10
    finally:
        g.close()
