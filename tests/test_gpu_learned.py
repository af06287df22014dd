"""The learned right preconditioner on the GPU against its FP64 restatement (oracle/net_oracle.py).

Tolerances (relative 2-norm errors):
  * graph: bit-exact (CSR, neighbour ids and periodic shift codes);
  * context features: within one bf16 rounding step of the oracle's (2^-8 relative per entry);
  * forward, against the oracle that rounds to bf16 where the kernels do: 2e-3 per hidden layer,
    decoder output and z -- what is left is FP32 (tensor-core) against FP64 accumulation and the
    rare bf16 rounding or relu flip it causes; against exact arithmetic (no bf16 anywhere): 5e-2,
    the error of the bf16 operands themselves;
  * gradients: 1e-3 per parameter block against the rounding oracle (observed 1e-7 to 1e-5 on
    a GB300), 1e-1 against exact arithmetic (the backward rounds the gradients of every GEMM operand
    to bf16).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import net_oracle as no
from phasta_gb300 import _lib as L
from phasta_gb300 import learn, mesh
from phasta_gb300.solver import GpuSolver, make_params

from helpers import rel

pytestmark = pytest.mark.gpu


def _mixed(case, ph, **kw):
    p = make_params(ph["mu"], ph["dt"], Kspace=20, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                    outer_residual=L.PHGPU_RES_SPLITDF, **kw)
    return GpuSolver(case, p), p


def _loc(v_ref, N):
    return np.ascontiguousarray(np.asarray(v_ref).reshape(5, N).T)


def _ref(v_loc):
    return np.ascontiguousarray(np.asarray(v_loc).T).reshape(-1)


def _y_loc(y_ref, N):
    y = np.asarray(y_ref).reshape(5, N)
    return np.stack([y[3], y[0], y[1], y[2], y[4]], axis=1)


def _bd_dev(bd_ref, N):
    return np.asarray(bd_ref).reshape(5, 5, N).transpose(2, 1, 0).reshape(N, 25)


def _random_weights(seed):
    rng = np.random.default_rng(seed)
    p = no.unpack(no.init_weights(seed, zero_decoder=False))
    for k in p:
        if k.startswith("b_"):
            p[k] = 0.1 * rng.standard_normal(p[k].shape)
    p["W_d"] *= 0.5
    p["alpha"] = 1.0 + 0.2 * rng.standard_normal(5)
    p["beta"] = 1.0 + 0.2 * rng.standard_normal(5)
    return no.pack(p)


@pytest.fixture(scope="module")
def chan(gpu_lib):
    case, ph = mesh.channel_case(6)
    g, p = _mixed(case, ph)
    y = mesh.uniform_state(case, 0.3, sigma=0.02)
    ac = np.zeros_like(y)
    _, bd, Dy, st = g.SolMFG(y, ac)
    return case, g, y, bd


@pytest.mark.parametrize("which", ["channel", "mixed"])
def test_graph_is_the_oracles(gpu_lib, which):
    if which == "channel":
        case, ph = mesh.channel_case(5)
    else:
        case, ph = mesh.mixed_case(3, 3, (3, 3, 2))
    g, _ = _mixed(case, ph)
    nstart, nbr, geo = g.net_graph()
    o = no.Graph(case)
    assert np.array_equal(nstart, o.start.astype(np.int32))
    assert np.array_equal(nbr.astype(np.int64), o.packed)
    assert np.allclose(geo[:3], o.L, rtol=1e-7, atol=0)
    assert abs(geo[3] - o.rh) <= 1e-6 * o.rh


def test_context_features(chan):
    case, g, y, bd = chan
    N = case.nshg
    f = g.net_features()
    act = no.active_mask(case)
    ref = no.context(no.f32(_bd_dev(bd, N)), _y_loc(y, N), act, g.params["Rgas"], g.params["gamma"])
    err = np.abs(f - ref)
    assert np.all(err <= 2.0 ** -7 * np.abs(ref) + 1e-30), float((err / (np.abs(ref) + 1e-30)).max())
    assert np.array_equal(f[:, 30], act)


def _vt(case, seed):
    rng = np.random.default_rng(seed)
    N = case.nshg
    act = no.active_mask(case)
    v = rng.standard_normal((N, 5)) * act[:, None]
    v /= np.linalg.norm(v)
    t = v + 0.5 * rng.standard_normal((N, 5)) * act[:, None] / np.sqrt(5 * N)
    return v, t, act


def test_forward_every_layer_matches_the_oracle(chan):
    case, g, y, bd = chan
    N = case.nshg
    w = _random_weights(11)
    g.net_set_weights(w)
    ctx = g.net_features().astype(np.float64)
    v, _, act = _vt(case, 3)
    z, hid, out = g.net_apply(_ref(v), hidden=True)
    G = no.Graph(case)
    ze, oute, ce = no.forward(w, G, v, ctx, act, emulate=True)
    zx, outx, cx = no.forward(w, G, v, ctx, act, emulate=False)
    errs = []
    for l in range(4):
        e = rel(hid[l], ce["h"][l])
        errs.append(e)
        assert e < 2e-3, (l, e)
        assert rel(hid[l], cx["h"][l]) < 5e-2, l
    assert rel(out[:, :5], oute) < 2e-3 and rel(out[:, :5], outx) < 5e-2
    zl = _loc(z, N)
    assert rel(zl - v, ze - v) < 2e-3 and rel(zl - v, zx - v) < 5e-2
    # inactive nodes (slaves, Dirichlet) pass v through unchanged
    assert np.array_equal(zl[act == 0], v[act == 0].astype(np.float32).astype(np.float64))
    print("hidden-layer errors vs the rounding oracle:", ["%.1e" % e for e in errs])


def test_gradients_match_the_oracle(chan):
    case, g, y, bd = chan
    N = case.nshg
    w = _random_weights(12)
    g.net_set_weights(w)
    ctx = g.net_features().astype(np.float64)
    v, t, act = _vt(case, 4)
    loss, grad = g.net_loss_grad(_ref(v), _ref(t))
    G = no.Graph(case)
    le, ge, _ = no.loss_grad(w, G, v, t, ctx, act, emulate=True)
    lx, gx, _ = no.loss_grad(w, G, v, t, ctx, act, emulate=False)
    assert abs(loss - le) <= 2e-3 * le and abs(loss - lx) <= 5e-2 * lx, (loss, le, lx)
    worst = {}
    for name, (o, s) in no.OFFSETS.items():
        n = int(np.prod(s))
        a, b, c = grad[o:o + n], ge[o:o + n], gx[o:o + n]
        if name in ("alpha", "beta"):
            assert not a.any()
            continue
        worst[name] = rel(a, b)
        assert rel(a, b) < 1e-3, (name, rel(a, b))
        assert rel(a, c) < 1e-1, (name, rel(a, c))
    print("gradient errors vs the rounding oracle:", {k: "%.1e" % e for k, e in worst.items()})


def test_training_on_the_gpu_lowers_the_loss(gpu_lib):
    case, ph = mesh.channel_case(8)
    g, _ = _mixed(case, ph)
    rep = learn.collect_pairs(g, case, 24, seed=5)
    assert rep["pairs"] == 24
    g.net_set_weights(learn.init_weights(5))
    tr = g.net_train(12, lr=2e-3, seed=5)
    assert tr["steps"] == 12 * 24
    assert np.isfinite(tr["loss_last"]) and tr["loss_last"] < 0.8 * tr["loss_first"], tr
    w = g.net_get_weights()
    assert np.all(np.isfinite(w)) and np.any(w[no.OFFSETS["W_d"][0]:no.OFFSETS["b_d"][0]] != 0)


def _solve(g, y, ac):
    _, _, Dy, st = g.SolMFG(y, ac)
    return Dy, st


def test_identity_network_falls_back_and_still_converges(gpu_lib):
    """A network that does nothing (zero decoder) cannot converge below the block-diagonal count:
    the solve falls back, converges anyway, and the network is switched off after two such
    failures, or after the first when that learned cycle took more than twice the time of the
    block-diagonal iterations it was to replace."""
    case, ph = mesh.channel_case(8)
    g, p = _mixed(case, ph, precond=L.PHGPU_PRECOND_LEARNED)
    y = mesh.uniform_state(case, 0.3, sigma=0.02)
    ac = np.zeros_like(y)
    g.net_set_weights(learn.init_weights(1))
    seen = []
    for _ in range(4):
        Dy, st = _solve(g, y, ac)
        assert st.echeck <= p["etol"] * st.unorm0 * (1 + 1e-12), st
        seen.append(st.net_fallback)
    assert seen in ([L.PHGPU_NET_PLAIN, L.PHGPU_NET_FELL_BACK, L.PHGPU_NET_FELL_BACK, L.PHGPU_NET_PLAIN],
                    [L.PHGPU_NET_PLAIN, L.PHGPU_NET_FELL_BACK, L.PHGPU_NET_PLAIN, L.PHGPU_NET_PLAIN]), seen
    u = g.net_usage()
    nfb = seen.count(L.PHGPU_NET_FELL_BACK)
    assert u["off"] and u["fell_back"] == nfb and u["plain"] == 4 - nfb
    # with the network off, a time step is block-diagonal and runs as one CUDA graph
    g.time_step(y, ac, 3)
    assert g.step_graphs == 1 and g.net_usage()["plain"] == 7 - nfb


def test_nonfinite_network_output_falls_back(gpu_lib):
    case, ph = mesh.channel_case(8)
    g, p = _mixed(case, ph, precond=L.PHGPU_PRECOND_LEARNED)
    y = mesh.uniform_state(case, 0.3, sigma=0.02)
    ac = np.zeros_like(y)
    w = learn.init_weights(2)
    o = no.OFFSETS["b_d"][0]
    w[o:o + 5] = 3e38  # the decoder's output overflows once scaled: the cycle goes non-finite
    g.net_set_weights(w)
    Dy0, st0 = _solve(g, y, ac)
    assert st0.net_fallback == L.PHGPU_NET_PLAIN
    Dy1, st1 = _solve(g, y, ac)
    assert st1.net_fallback == L.PHGPU_NET_FELL_BACK
    assert np.all(np.isfinite(Dy1)) and st1.echeck <= p["etol"] * st1.unorm0 * (1 + 1e-12)
    assert rel(Dy1, Dy0) < 1e-2


def test_learned_cycle_graph_equals_launched_cycle(gpu_lib):
    case, ph = mesh.channel_case(8)
    y = mesh.uniform_state(case, 0.3, sigma=0.02)
    ac = np.zeros_like(y)
    w = _random_weights(13)
    o = no.OFFSETS["W_d"][0]
    w[o:o + 5 * 64] *= 0.05
    out = []
    for no_graph in (0, 1):
        g, p = _mixed(case, ph, precond=L.PHGPU_PRECOND_LEARNED)
        g.set_params(no_graph=no_graph)
        g.net_set_weights(w)
        _solve(g, y, ac)  # the block-diagonal reference count
        Dy, st = _solve(g, y, ac)
        out.append((Dy, st))
        if no_graph == 0:
            assert g.graph_cycles >= 1
    (d0, s0), (d1, s1) = out
    # the same cycles in the same order (whether the cycle counts as a gain is a timing verdict)
    assert s0.net_its == s1.net_its and s0.iKs == s1.iKs
    assert np.array_equal(d0, d1)


def test_trained_network_in_flexible_gmres(gpu_lib):
    """Train on pairs of a 12^3 x 6 channel, then solve a 16^3 x 6 channel (the CPU-sized case of the
    benchmark definitions) with and without the network: both reach the Krylov tolerance; the
    iteration counts are reported."""
    case_t, ph_t = mesh.channel_case(12)
    gt, _ = _mixed(case_t, ph_t)
    w, rep = learn.train(gt, case_t, n_pairs=96, epochs=10, lr=2e-3, seed=7)
    assert rep["train"]["loss_last"] < rep["train"]["loss_first"], rep
    case, ph = mesh.channel_case(16)
    y = mesh.uniform_state(case, 0.3, sigma=0.01)
    ac = np.zeros_like(y)
    g, p = _mixed(case, ph, precond=L.PHGPU_PRECOND_LEARNED)
    g.net_set_weights(w)
    Dy0, st0 = _solve(g, y, ac)
    Dy1, st1 = _solve(g, y, ac)
    for st in (st0, st1):
        assert st.echeck <= p["etol"] * st.unorm0 * (1 + 1e-12)
    assert st0.net_fallback == L.PHGPU_NET_PLAIN
    assert rel(Dy1, Dy0) < 5e-2
    print(f"block-diagonal GMRES {st0.iKs} iterations; learned flexible GMRES {st1.net_its} "
          f"({'used' if st1.net_fallback == 0 else 'fell back'}), loss {rep['train']['loss_first']:.3e} -> "
          f"{rep['train']['loss_last']:.3e}")
