"""Contexts used from several host threads at once.

Each context owns its stream, buffers and graphs; what the library shares between contexts
(the constant-memory tables, identical for all) is written with the same values by every
create, and the CUDA graphs are captured in relaxed mode, so another thread's allocations
and copies do not disturb a capture.  Two contexts driven from two threads at the same time
(ctypes releases the interpreter lock during each call) give bitwise the results of the same
runs one after the other: creates, autotuned mixed-precision time steps with step graphs,
and the FP64 path."""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from helpers import channel, layered, mixed
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


def _run(job):
    case, p, y, ac = job
    g = GpuSolver(case, p)
    try:
        g.set_tuning(4, 3)
        out = []
        for _ in range(2):
            _yo, _ao, y, ac, st = g.time_step(y, ac, nitr=2)
            out.append((y.copy(), ac.copy(), st.iKs))
        return out
    finally:
        g.close()


def _jobs():
    mx = dict(precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF)
    jobs = []
    for make in (lambda: channel(12, ac_scale=0.05, Kspace=20), lambda: mixed(4, 4, (4, 4, 2), Kspace=20),
                 lambda: layered(5, (2, 1, 2), Kspace=20)):
        case, p, y, ac = make()
        jobs.append((case, dict(p, **mx), y, ac))
    case, p, y, ac = channel(8, ac_scale=0.05)
    jobs.append((case, p, y, ac))  # FP64, finite-difference product
    return jobs


def test_contexts_on_several_threads_match_sequential_runs(gpu_lib):
    jobs = _jobs()
    ref = [_run(j) for j in jobs]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        got = list(ex.map(_run, jobs))
    for r, g in zip(ref, got):
        for (ya, aa, ka), (yb, ab, kb) in zip(r, g):
            assert ka == kb
            assert np.array_equal(ya, yb) and np.array_equal(aa, ab)


def test_the_same_mesh_on_two_threads(gpu_lib):
    job = _jobs()[0]
    ref = _run(job)
    with ThreadPoolExecutor(max_workers=2) as ex:
        got = list(ex.map(_run, [job, job]))
    for g in got:
        for (ya, aa, ka), (yb, ab, kb) in zip(ref, g):
            assert ka == kb and np.array_equal(ya, yb) and np.array_equal(aa, ab)
