"""GPU runs started from PHASTA files: geombc + restart in, restart out, checkphasta.

The benchmark meshes are written as geombc.dat.1 and restart.0.1, read back through
the library's readers (geniBC, genBC1), run for two time steps on the GPU and written
as restart.<step>.1; checkphasta's comparison with the same run started from the
in-memory arrays must find no difference at all (the GPU path is deterministic).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import channel, layered, mixed
from phasta_gb300 import _lib as L
from phasta_gb300 import phio
from phasta_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


def _run(case, p, y, ac, out, steps=2):
    out.mkdir()
    g = GpuSolver(case, p)
    try:
        for step in range(1, steps + 1):
            _yo, _ao, y, ac, _st = g.time_step(y, ac, nitr=2)
            phio.write_restart(out, step, y.reshape(5, -1), ac.reshape(5, -1))
    finally:
        g.close()
    return y


@pytest.mark.parametrize("make,precision", [
    (lambda: channel(8, ac_scale=0.05, Kspace=10), L.PHGPU_FP64),
    (lambda: channel(8, ac_scale=0.05, Kspace=10), L.PHGPU_MIXED),
    (lambda: mixed(3, 3, (3, 3, 2), Kspace=10), L.PHGPU_MIXED),
    (lambda: layered(4, (2, 1, 2), periodic_x=False, Kspace=10), L.PHGPU_MIXED),
], ids=["channel8-fp64", "channel8-mixed", "mixed3-mixed", "layered-open-mixed"])
def test_run_from_phasta_files(tmp_path, make, precision):
    case, p, y, ac = make()
    p = dict(p, precision=precision, ap_mode=L.PHGPU_AP_LINEAR if precision == L.PHGPU_MIXED else L.PHGPU_AP_FD)
    run = tmp_path / "run"
    run.mkdir()
    phio.write_case(case, run)
    phio.write_restart(run, 0, y.reshape(5, -1), ac.reshape(5, -1))
    case2 = phio.read_case(run)
    y2, ac2, lstep = phio.read_restart(run, 0, case2.nshg)
    assert lstep == 0 and np.array_equal(y2.reshape(-1), y) and np.array_equal(ac2.reshape(-1), ac)
    ya = _run(case, p, y, ac, tmp_path / "a")
    yb = _run(case2, p, y2.reshape(-1), ac2.reshape(-1), tmp_path / "b")
    assert np.all(np.isfinite(ya)) and not np.array_equal(ya, y)
    m, n, ok = phio.checkphasta(tmp_path / "a", tmp_path / "b", 0.0)
    assert n == 2 and m == 0.0 and ok


@pytest.mark.parametrize("make", [
    lambda: channel(8, ac_scale=0.05, Kspace=10),
    lambda: layered(4, (2, 1, 2), periodic_x=False, Kspace=10),
], ids=["channel8", "layered-open"])
def test_checkpoint_and_resume_is_bitwise_the_uninterrupted_run(tmp_path, make):
    """checkpoint (restar('out ') of yold/acold after itrUpdate) at step 2 of a four-step run; a
    new context started from that restart file (restar('in  ')) runs steps 3 and 4: bitwise the
    uninterrupted run's state.  Mixed precision with the linearized product: the restart's
    state is all that a time step carries from one step to the next."""
    case, p, y, ac = make()
    p = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF)
    ck = tmp_path / "ck"
    ck.mkdir()
    g = GpuSolver(case, p)
    try:
        g.set_tuning(4, 3)
        for step in range(1, 5):
            _yo, _ao, y, ac, _st = g.time_step(y, ac, nitr=2)
            if step == 2:
                phio.write_restart(ck, 2, y.reshape(5, -1), ac.reshape(5, -1))
    finally:
        g.close()
    yr, acr, lstep = phio.read_restart(ck, 2, case.nshg)
    assert lstep == 2
    yr, acr = yr.reshape(-1), acr.reshape(-1)
    g2 = GpuSolver(case, p)
    try:
        g2.set_tuning(4, 3)
        for _ in range(2):
            _yo, _ao, yr, acr, _st = g2.time_step(yr, acr, nitr=2)
    finally:
        g2.close()
    assert np.array_equal(yr, y) and np.array_equal(acr, ac)
