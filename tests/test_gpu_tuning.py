"""Autotuned variants of the pipelined element sweeps (phgpu_set_tuning / phgpu_tuning).

The linearized product is compiled for at least 3 or 4 resident CTAs per SM, the double-float
split residual for 2, 3 or 4: the same code under different register budgets.  A context times
them on its own mesh before its first mixed-precision matrix-free solve and keeps the fastest;
every forced choice must give bit for bit the same time steps."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import channel
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


def _run(case, p, y, ac, force=None, nsteps=2):
    g = GpuSolver(case, p)
    try:
        if force is not None:
            g.set_tuning(*force)
        out = []
        for _ in range(nsteps):
            _yo, _ao, y, ac, st = g.time_step(y, ac, nitr=2)
            out.append((y.copy(), ac.copy(), st.iKs, g.ntotGM))
        return out, g.tuning(), g.kernel_launches
    finally:
        g.close()


@pytest.mark.parametrize("no_graph", [0, 1], ids=["step-graph", "launched"])
def test_forced_variants_give_bitwise_the_same_steps(no_graph):
    case, p, y, ac = channel(10, ac_scale=0.05, Kspace=20)
    p = dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF,
             no_graph=no_graph)
    ref, tun, launches = _run(case, p, y, ac)
    assert tun["how"] == "tuned"
    assert tun["lin_minb"] in (3, 4) and tun["ress_minb"] in (2, 3, 4)
    assert all(t > 0 for t in tun["lin_ms"].values()) and all(t > 0 for t in tun["ress_ms"].values())
    # the chosen variant is the fastest one timed
    assert tun["lin_ms"][tun["lin_minb"]] == min(tun["lin_ms"].values())
    assert tun["ress_ms"][tun["ress_minb"]] == min(tun["ress_ms"].values())
    for force in [(3, 2), (4, 4), (3, 3), (4, 2)]:
        got, t2, l2 = _run(case, p, y, ac, force=force)
        assert t2["how"] == "forced" and (t2["lin_minb"], t2["ress_minb"]) == force
        assert l2 == launches  # tuning launches are not counted
        for (ya, aa, ka, na), (yb, ab, kb, nb) in zip(ref, got):
            assert np.array_equal(ya, yb) and np.array_equal(aa, ab) and ka == kb and na == nb


def test_set_tuning_checks_its_arguments_and_resets():
    case, p, y, ac = channel(6, ac_scale=0.05)
    g = GpuSolver(case, dict(p, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR))
    try:
        assert g.tuning()["how"] == "default"
        with pytest.raises(RuntimeError):
            g.set_tuning(5, 3)
        with pytest.raises(RuntimeError):
            g.set_tuning(3, 1)
        g.set_tuning(3, 2)
        assert g.tuning()["how"] == "forced"
        g.set_tuning(0, 0)
        assert g.tuning()["how"] == "default"
        g.time_step(y, ac, nitr=1)
        t = g.tuning()
        assert t["how"] == "tuned"
        # the split residual is timed only when it is the outer residual in use
        split = p.get("outer_residual", 0) == L.PHGPU_RES_SPLITDF
        assert all((v > 0) == split for v in t["ress_ms"].values())
    finally:
        g.close()
