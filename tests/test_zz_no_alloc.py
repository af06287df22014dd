"""GPU test of phgpu_rstat_noalloc, the allocation-free residual statistic.

phgpu_rstat_noalloc serves callers that cannot allocate device memory (a host
code whose device memory is owned by its own pool or by another framework's
allocator): they pass a device residual and a device result slot, and the
entry point works in a fixed static device array of the library.  Here the
test plays that caller: it owns the buffers (allocated through torch) and
checks the statistic against phgpu_stats.totres of phgpu_solmfg, which computes
sqrt(sum res^2)/nshg of the same L^-1 R with the context's own reduction.
Tolerance: 1e-12 relative (FP64 sums in a different order).  Two calls in a row
must both agree, which shows that the shared array's leftover contents from the
previous call do not leak into the next.  This file is collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import channel
from phasta_gb300 import _lib as L
from phasta_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(lib, res_dev, nshg, out_dev, stream):
    return lib.phgpu_rstat_noalloc(C.c_void_p(res_dev.data_ptr()), nshg, C.c_void_p(out_dev.data_ptr()),
                                   C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("n", [16, 32])
def test_rstat_noalloc_matches_solmfg_totres_on_two_calls_in_a_row(gpu_lib, n):
    import torch
    case, p, y, ac = channel(n, ac_scale=0.05)
    g = GpuSolver(case, p)
    res, _, _, st = g.SolMFG(y, ac)
    totres = st.totres
    nshg = case.nshg
    assert totres > 0.0 and res.size == 5 * nshg

    res_dev = torch.from_numpy(np.ascontiguousarray(res)).to("cuda:0")
    out_dev = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream()
    assert _noalloc(gpu_lib, res_dev, nshg, out_dev[0:1], stream) == L.PHGPU_OK
    assert _noalloc(gpu_lib, res_dev, nshg, out_dev[1:2], stream) == L.PHGPU_OK
    torch.cuda.synchronize()
    got = out_dev.cpu().numpy()
    assert np.all(np.abs(got - totres) <= TOL * totres), (got, totres)


def test_rstat_noalloc_after_a_larger_call_and_rejections(gpu_lib):
    import torch
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(5)
    out_dev = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    # a large call fills many block partials, then a small one must ignore them
    nshg_max = L.PHGPU_RSTAT_NOALLOC_MAX_N // 5  # the largest accepted nshg
    big = rng.standard_normal(5 * nshg_max)
    small = rng.standard_normal(5 * 1000)
    big_dev = torch.from_numpy(big).to("cuda:0")
    small_dev = torch.from_numpy(small).to("cuda:0")
    assert _noalloc(gpu_lib, big_dev, nshg_max, out_dev[0:1], stream) == L.PHGPU_OK
    assert _noalloc(gpu_lib, small_dev, 1000, out_dev[1:2], stream) == L.PHGPU_OK
    torch.cuda.synchronize()
    got = out_dev.cpu().numpy()
    want = np.array([np.sqrt(np.dot(big, big)) / nshg_max, np.sqrt(np.dot(small, small)) / 1000])
    # numpy sums 33.5M squares in another order: 1e-10 relative
    assert np.all(np.abs(got - want) <= 1e-10 * want), (got, want)
    # sizes beyond the fixed array and bad arguments are refused before any launch
    too_many = nshg_max + 1
    assert _noalloc(gpu_lib, big_dev, too_many, out_dev[0:1], stream) == L.PHGPU_ERR_TOO_LARGE
    assert gpu_lib.phgpu_rstat_noalloc(None, 1000, C.c_void_p(out_dev.data_ptr()), None) == L.PHGPU_ERR_INVALID
    assert _noalloc(gpu_lib, small_dev, 0, out_dev[0:1], stream) == L.PHGPU_ERR_INVALID
