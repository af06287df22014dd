"""The learned preconditioner's FP64 restatement (oracle/net_oracle.py), on the CPU.

The network has no reference implementation, so its oracle is pinned by its own
finite differences (central, FP64, no bf16 emulation) and by invariants of the
mesh graph."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import net_oracle as no
from phasta_gb300 import mesh


def _problem(case, seed=3):
    g = no.Graph(case)
    rng = np.random.default_rng(seed)
    N = case.nshg
    act = no.active_mask(case)
    v = rng.standard_normal((N, 5)) * act[:, None]
    v /= np.linalg.norm(v)
    t = v + 0.3 * rng.standard_normal((N, 5)) / np.sqrt(5 * N)
    ctx = no.bf16(rng.standard_normal((N, no.F_CTX)))
    ctx[:, 30] = act
    w = no.init_weights(seed, zero_decoder=False)
    p = no.unpack(w)
    for k in p:
        if k.startswith("b_"):
            p[k] = 0.1 * rng.standard_normal(p[k].shape)
    p["alpha"] = 1.0 + 0.2 * rng.standard_normal(5)
    p["beta"] = 1.0 + 0.2 * rng.standard_normal(5)
    return g, no.pack(p).astype(np.float64), v, t, ctx, act


def test_graph_is_symmetric_with_consistent_edge_vectors():
    case, _ = mesh.channel_case(4)
    g = no.Graph(case)
    fwd = {(int(s), int(d), int(c)) for s, d, c in zip(g.src, g.dst, g.code)}
    flip = {1: 2, 2: 1, 0: 0}
    for s, d, c in list(fwd)[:500]:
        nc = sum(flip[(c >> (2 * k)) & 3] << (2 * k) for k in range(3))
        assert (d, s, nc) in fwd
    # interior nodes of the Kuhn split have 14 neighbours; periodic y/z wrap keeps that on the masters
    iper = case.iper
    masters = np.where(iper == np.arange(case.nshg))[0]
    x = case.x[masters, 0]
    inner = masters[(x > 1e-12) & (x < 1 - 1e-12)]
    assert np.all(g.deg[inner] == 14)
    assert np.all(g.deg[iper != np.arange(case.nshg)] == 0)   # slaves are isolated
    # edge vectors are the element edges' own geometry (no periodic jump of length ~1)
    assert np.abs(g.vec_true).max() <= case.h * 1.0000001
    assert np.allclose(g.e / g.rh, g.vec_true, atol=1e-6)


def test_graph_of_hexes_and_wedges():
    case, _ = mesh.mixed_case(3, 3, (3, 3, 2))
    g = no.Graph(case)
    assert g.src.size > 0 and np.all(np.bincount(g.src, minlength=case.nshg) == g.deg)
    # hex edges only (no face diagonals): 6 neighbours per periodic hex node
    nt = 4 ** 3
    nh = 4 ** 3
    hex_nodes = np.arange(nt, nt + nh)
    hm = hex_nodes[case.iper[hex_nodes] == hex_nodes]
    assert np.all(g.deg[hm] == 6)


@pytest.mark.parametrize("which", ["channel", "mixed"])
def test_backward_matches_finite_differences(which):
    if which == "channel":
        case, _ = mesh.channel_case(3)
    else:
        case, _ = mesh.mixed_case(2, 2, (2, 2, 2))
    g, w, v, t, ctx, act = _problem(case)
    loss, grad, _ = no.loss_grad(w, g, v, t, ctx, act, emulate=False)
    rng = np.random.default_rng(7)
    train = np.arange(no.NTRAIN)
    for trial in range(4):
        d = np.zeros(no.NPARAM)
        d[train] = rng.standard_normal(no.NTRAIN)
        eps = 1e-8
        lp = no.loss_grad(w + eps * d, g, v, t, ctx, act, emulate=False)[0]
        lm = no.loss_grad(w - eps * d, g, v, t, ctx, act, emulate=False)[0]
        fd = (lp - lm) / (2 * eps)
        an = float(grad @ d)
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-8), (trial, fd, an)
    # per-block check: each parameter block's directional derivative alone
    for name, (o, sh) in no.OFFSETS.items():
        if name in ("alpha", "beta"):
            continue
        d = np.zeros(no.NPARAM)
        n = int(np.prod(sh))
        d[o:o + n] = rng.standard_normal(n)
        eps = 1e-8
        fd = (no.loss_grad(w + eps * d, g, v, t, ctx, act, emulate=False)[0] -
              no.loss_grad(w - eps * d, g, v, t, ctx, act, emulate=False)[0]) / (2 * eps)
        an = float(grad @ d)
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-9) + 1e-12, (name, fd, an)


def test_emulated_rounding_stays_close_to_exact():
    case, _ = mesh.channel_case(3)
    g, w, v, t, ctx, act = _problem(case)
    l0, g0, z0 = no.loss_grad(w, g, v, t, ctx, act, emulate=False)
    l1, g1, z1 = no.loss_grad(w, g, v, t, ctx, act, emulate=True)
    assert abs(l1 - l0) <= 2e-2 * l0
    assert np.linalg.norm(g1 - g0) <= 5e-2 * np.linalg.norm(g0)
    assert np.linalg.norm(z1 - z0) <= 2e-2 * np.linalg.norm(z0 - v)


def test_zero_decoder_is_the_identity():
    case, _ = mesh.channel_case(3)
    g, _, v, t, ctx, act = _problem(case)
    w = no.init_weights(1, zero_decoder=True)
    z, out, _ = no.forward(w, g, v, ctx, act)
    assert np.array_equal(z, v) and not out.any()


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e38, 1e-40])
    r = no.bf16(vals)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 4 * 2 ** -8 and r[3] == 1.0 and r[4] == -2.5
    assert np.isfinite(r[5])
