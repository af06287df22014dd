"""Reverse Cuthill-McKee node order (phgpu_rcm_order, host code: no GPU needed)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import channel
from oracle import pyoracle
from phasta_gb300 import mesh
from phasta_gb300.solver import rcm_order


def _shuffled(case, seed=5):
    p = np.random.default_rng(seed).permutation(case.nshg)
    return mesh.renumber(case, p), p


@pytest.mark.parametrize("which", ["channel", "layered", "mixed"])
def test_rcm_is_a_permutation_that_restores_a_narrow_band(gpu_lib, which):
    case = {"channel": lambda: mesh.channel_case(10)[0],
            "layered": lambda: mesh.layered(10, 4, 2, 6),
            "mixed": lambda: mesh.mixed_case(6, 6, (6, 6, 3))[0]}[which]()
    shuf, _ = _shuffled(case)
    p, bw_before, bw_after = rcm_order(shuf)
    assert np.array_equal(np.sort(p), np.arange(case.nshg))
    _, _, bw_rcm_nat = rcm_order(case)
    assert bw_before > 0.5 * case.nshg            # a random order has a band as wide as the mesh
    assert bw_after <= 0.4 * case.nshg            # RCM narrows it to a few cross-sections
    assert bw_after <= 1.5 * bw_rcm_nat           # whatever order the nodes came in
    # deterministic
    p2, _, _ = rcm_order(shuf)
    assert np.array_equal(p, p2)


def test_rcm_keeps_periodic_pairs_close(gpu_lib):
    case = mesh.channel_case(6)[0]
    shuf, _ = _shuffled(case, seed=9)
    p, _, bw = rcm_order(shuf)
    r = mesh.renumber(shuf, p)
    slaves = np.where(r.iper != np.arange(r.nshg))[0]
    assert slaves.size > 0 and np.abs(slaves - r.iper[slaves]).max() <= bw


def test_renumbered_mesh_gives_the_renumbered_residual():
    """The oracle's ElmMFG is equivariant under the renumbering (the mesh helpers are consistent)."""
    case, p, y, ac = channel(3, ac_scale=0.05)
    perm = np.random.default_rng(2).permutation(case.nshg)
    r = mesh.renumber(case, perm)
    res_a, rmes_a, bd_a = pyoracle.Oracle(case, p).ElmMFG(y, ac)
    res_b, rmes_b, bd_b = pyoracle.Oracle(r, p).ElmMFG(mesh.renumber_field(y, perm, 5),
                                                        mesh.renumber_field(ac, perm, 5))
    for a, b, nc in ((res_a, res_b, 5), (rmes_a, rmes_b, 5), (bd_a, bd_b, 25)):
        assert np.abs(mesh.renumber_field(a, perm, nc) - b).max() <= 1e-12 * np.abs(a).max()


def test_rcm_rejects_out_of_range_connectivity(gpu_lib):
    case = mesh.channel_case(3)[0]
    case.ien[0, 0] = case.nshg
    with pytest.raises(RuntimeError):
        rcm_order(case)
