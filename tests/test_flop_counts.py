"""The oracle's element routine with a counting scalar (oracle/count_flops.py): the counted
instance computes the same element outputs as the oracle (the count follows the oracle's
statements), and profiles/flops_per_element.json is what the counter gives."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from helpers import channel, layered
from oracle import count_flops as cf


@pytest.mark.parametrize("lcsyst", [1, 2, 3])
@pytest.mark.parametrize("mode", list(cf.MODES))
def test_counting_instance_computes_the_oracles_outputs(lcsyst, mode):
    if lcsyst == 1:
        case, p, y, ac = channel(4, ac_scale=0.05)
    else:
        case, p, y, ac = layered(3, (1, 1, 1))
    ires, iprec = cf.MODES[mode]
    nf, out, ref = cf.count(p, lcsyst, ires, iprec, *cf.element_arrays(case, y, ac, lcsyst))
    assert nf > 1000
    for a, b in zip(out, ref):
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(b).max()))


def test_committed_counts_are_current(tmp_path):
    doc = cf.main(tmp_path / "f.json")
    committed = json.loads((Path(__file__).resolve().parents[1] / "profiles" / "flops_per_element.json").read_text())
    assert committed["per_element"] == doc["per_element"]
    t = doc["per_element"]["tet"]
    assert t["bdiag"] > 0.7 * t["full"] and 4000 < t["res"] < 8000
