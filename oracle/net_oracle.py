"""FP64 restatement of the learned preconditioner's network -- test infrastructure only.

Only tests/ and the smoke check import this module, as the checker of the GPU
network kernels (phasta_gb300/csrc/learn.cu); nothing in the product path
calls it.

The network has no counterpart in the reference (PHASTA preconditions its
matrix-free GMRES with the 5x5 block-diagonal LU only: solmfg.f:221-340 calls
i3LU, i3lu.f:125-148).  It is a right preconditioner of the block-diagonal
preconditioned operator A~ = L^-1 J U^-1 that SolMFG's Krylov loop multiplies
by (au1mfg.f:57-83), used inside flexible GMRES.  Its definition, restated
here and implemented by the kernels:

  graph    the mesh edges of every element block (tet 6, hex 12, wedge 9
           edges), mapped to periodic masters (iper); per directed edge
           i -> j the edge vector e_ij = (x_b - x_a) / hbar of the element
           edge it came from (periodic wrap kept), hbar the mean edge length
  input    x_i = [ ctx_i (32) | s alpha_d v_i,d (5) | 0 (11) ]        bf16
           s = sqrt(5 nshg) (v has unit 2-norm, so s v_i is O(1) per node)
           ctx_i = 25 entries of node i's factored BDiag block over their
           RMS, 10 (p/pbar - 1), u/cbar, v/cbar, w/cbar, 10 (T/Tbar - 1),
           active flag, 0
  encoder  h0 = bf16(relu(W_e x + b_e))                    W_e: 64 x 48
  layer l  P = bf16(W_p h), Q = W_q h + b_m                W_p, W_q: 64 x 64
           m_ij = relu(Q_i + P_j + C e_ij)                 C: 64 x 3
           a_i = bf16(sum_j m_ij / deg_i)
           u = W_u [h; a] + b_u,  h' = bf16(h + relu(u))   W_u: 64 x 128
  decoder  out = W_d h3 + b_d                              W_d: 5 x 64
  output   z_i,d = v_i,d + act_i beta_d out_i,d / s

GEMM weights enter as bf16 (round to nearest even); biases, C and the
normalisation constants alpha, beta are FP32.  With ``emulate=True`` the
forward and backward round to bf16 at exactly the points the kernels do, so
the only remaining difference is FP32 vs FP64 accumulation; with
``emulate=False`` it is the network in exact arithmetic (the gradient the
bf16 training approximates).

Training pairs (v, t): v = A~ w / ||A~ w||, t = w / ||A~ w|| for w the plain
block-diagonal GMRES solution; the loss is the masked mean square of
out - s (t - v) / beta over the 5 dofs of the active nodes.

Parity of this restatement is pinned by finite differences of its own loss
(tests/test_net_oracle.py): the network has no reference implementation.
"""
from __future__ import annotations

import math

import numpy as np

H = 64          # hidden width
F_IN = 48       # input features (32 context + 5 direction + 11 zero)
F_CTX = 32
NL = 3          # message-passing layers
NOUT = 5

# flat parameter layout (FP32), shared with include/phgpu.h
_LAYOUT = [("W_e", (H, F_IN)), ("b_e", (H,))]
for _l in range(NL):
    _LAYOUT += [(f"W_p{_l}", (H, H)), (f"W_q{_l}", (H, H)), (f"b_m{_l}", (H,)), (f"C{_l}", (H, 3)),
                (f"W_u{_l}", (H, 2 * H)), (f"b_u{_l}", (H,))]
_LAYOUT += [("W_d", (NOUT, H)), ("b_d", (NOUT,)), ("alpha", (NOUT,)), ("beta", (NOUT,))]
OFFSETS = {}
_o = 0
for _n, _s in _LAYOUT:
    OFFSETS[_n] = (_o, _s)
    _o += int(np.prod(_s))
NPARAM = _o
NTRAIN = NPARAM - 2 * NOUT   # alpha and beta are normalisation constants, not trained
GEMM_WEIGHTS = {"W_e", "W_d"} | {f"W_{k}{l}" for k in "pqu" for l in range(NL)}


def unpack(w: np.ndarray) -> dict:
    w = np.asarray(w, dtype=np.float64)
    return {n: w[o:o + int(np.prod(s))].reshape(s) for n, (o, s) in OFFSETS.items()}


def pack(p: dict) -> np.ndarray:
    w = np.zeros(NPARAM, dtype=np.float32)
    for n, (o, s) in OFFSETS.items():
        w[o:o + int(np.prod(s))] = np.asarray(p[n], dtype=np.float32).reshape(-1)
    return w


def init_weights(seed: int = 1, zero_decoder: bool = True) -> np.ndarray:
    """He-scaled normal GEMM weights, zero biases; the decoder starts at zero so that the
    untrained preconditioner is the identity (plain block-diagonal GMRES)."""
    g = np.random.default_rng(seed)
    p = {}
    for n, (_, s) in OFFSETS.items():
        if n.startswith("W_"):
            fan_in = s[1]
            p[n] = g.standard_normal(s) * math.sqrt(2.0 / fan_in)
        elif n.startswith("C"):
            p[n] = g.standard_normal(s) * 0.5
        else:
            p[n] = np.zeros(s)
    p["W_u0"] *= 0.5
    p["W_u1"] *= 0.5
    p["W_u2"] *= 0.5
    if zero_decoder:
        p["W_d"][:] = 0.0
    p["alpha"] = np.ones(NOUT)
    p["beta"] = np.ones(NOUT)
    return pack(p)


# ---------------------------------------------------------------------------
# bf16 rounding (round to nearest even of the FP32 value, as __float2bfloat16_rn)
# ---------------------------------------------------------------------------
def bf16(a) -> np.ndarray:
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    nan = np.isnan(f)
    if nan.any():
        out = np.where(nan, f, out)
    return out.astype(np.float64)


def f32(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32).astype(np.float64)


# ---------------------------------------------------------------------------
# graph of the mesh edges
# ---------------------------------------------------------------------------
TET_EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
HEX_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
WEDGE_EDGES = [(0, 1), (1, 2), (2, 0), (3, 4), (4, 5), (5, 3), (0, 3), (1, 4), (2, 5)]
SHIFT_BITS = 26


class Graph:
    """CSR of directed edges between periodic masters, ascending (neighbour, shift code) per node."""

    def __init__(self, case):
        x = np.asarray(case.x, dtype=np.float64)
        iper = np.asarray(case.iper, dtype=np.int64)
        N = case.nshg
        a_list, b_list = [], []
        for conn, edges in ((case.ien, TET_EDGES), (case.ienh, HEX_EDGES), (case.ienw, WEDGE_EDGES)):
            conn = np.asarray(conn, dtype=np.int64)
            if conn.shape[0] == 0:
                continue
            for (p, q) in edges:
                a_list.append(conn[:, p])
                b_list.append(conn[:, q])
        a = np.concatenate(a_list)
        b = np.concatenate(b_list)
        i, j = iper[a], iper[b]
        keep = i != j
        a, b, i, j = a[keep], b[keep], i[keep], j[keep]
        dtrue = x[b] - x[a]
        diff = dtrue - (x[j] - x[i])
        L = np.abs(diff).max(axis=0) if diff.shape[0] else np.zeros(3)
        k = np.zeros_like(diff, dtype=np.int64)
        for d in range(3):
            if L[d] > 0:
                k[:, d] = np.rint(diff[:, d] / L[d]).astype(np.int64)
        assert np.all(np.abs(diff - k * L) <= 1e-9 * np.maximum(L, 1.0)), "non-translational periodicity"
        assert np.all(np.abs(k) <= 1)
        code = np.zeros(len(i), dtype=np.int64)
        for d in range(3):
            code |= np.where(k[:, d] == 1, 1, np.where(k[:, d] == -1, 2, 0)) << (2 * d)
        neg = np.zeros_like(code)
        for d in range(3):
            c = (code >> (2 * d)) & 3
            neg |= np.where(c == 1, 2, np.where(c == 2, 1, 0)) << (2 * d)
        src = np.concatenate([i, j])
        dst = np.concatenate([j, i])
        cod = np.concatenate([code, neg])
        vec = np.concatenate([dtrue, -dtrue])
        key = (src << 32) | (dst << 6) | cod
        key_u, first = np.unique(key, return_index=True)
        self.src = src[first]
        self.dst = dst[first]
        self.code = cod[first]
        self.vec_true = vec[first]
        self.N = N
        self.deg = np.bincount(self.src, minlength=N).astype(np.int64)
        self.start = np.concatenate([[0], np.cumsum(self.deg)]).astype(np.int64)
        self.L = L
        self.hbar = float(np.linalg.norm(self.vec_true, axis=1).mean()) if len(self.src) else 1.0
        self.packed = (self.dst | (self.code << SHIFT_BITS)).astype(np.int64)
        # edge vectors as the kernels form them: FP32 coordinates, FP32 shift and scale
        xf = f32(x)
        Lf = f32(L)
        sh = np.stack([np.where(((self.code >> (2 * d)) & 3) == 1, 1.0, np.where(((self.code >> (2 * d)) & 3) == 2,
                                                                                  -1.0, 0.0)) for d in range(3)], 1)
        rh = float(np.float32(1.0 / self.hbar))
        self.rh = rh
        self.e = (xf[self.dst] - xf[self.src] + sh * Lf) * rh


def active_mask(case) -> np.ndarray:
    """Nodes the network corrects: periodic masters without a Dirichlet bit (bits 0-5)."""
    iper = np.asarray(case.iper)
    return ((iper == np.arange(case.nshg)) & ((np.asarray(case.iBC) & 63) == 0)).astype(np.float64)


# ---------------------------------------------------------------------------
# context features
# ---------------------------------------------------------------------------
def context(bdf: np.ndarray, y_loc: np.ndarray, act: np.ndarray, Rgas: float, gamma: float) -> np.ndarray:
    """ctx (N, 32), bf16-rounded.  bdf: (N, 25) FP32 factored BDiag blocks (device layout,
    row-major 5x5); y_loc: (N, 5) state in (p, u, v, w, T) order; act: (N,) 0/1."""
    bdf = f32(bdf)
    na = max(act.sum(), 1.0)
    rms = np.sqrt((act[:, None] * bdf * bdf).sum(axis=0) / na)
    rms = np.where(rms > 0, rms, 1.0)
    pbar = (act * y_loc[:, 0]).sum() / na
    Tbar = (act * y_loc[:, 4]).sum() / na
    cbar = math.sqrt(gamma * Rgas * Tbar)
    ctx = np.zeros((bdf.shape[0], F_CTX))
    ctx[:, :25] = bdf / f32(rms)
    ctx[:, 25] = 10.0 * (y_loc[:, 0] / pbar - 1.0)
    ctx[:, 26:29] = y_loc[:, 1:4] / cbar
    ctx[:, 29] = 10.0 * (y_loc[:, 4] / Tbar - 1.0)
    ctx[:, 30] = act
    return bf16(ctx)


# ---------------------------------------------------------------------------
# forward / backward
# ---------------------------------------------------------------------------
def _relu(a):
    return np.maximum(a, 0.0)


def forward(w, g: Graph, v: np.ndarray, ctx: np.ndarray, act: np.ndarray, emulate: bool = True):
    """v: (N, 5) unit-norm direction in device dof order.  Returns (z, out, cache)."""
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    r32 = f32 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    p = unpack(w)
    Wg = {n: (r(p[n]) if n in GEMM_WEIGHTS else r32(p[n])) for n in p}
    N = v.shape[0]
    s = math.sqrt(5.0 * N)
    x = np.zeros((N, F_IN))
    x[:, :F_CTX] = ctx
    x[:, F_CTX:F_CTX + 5] = r(s * v * Wg["alpha"][None, :])
    pre_e = x @ Wg["W_e"].T + Wg["b_e"]
    h = r(_relu(pre_e))
    cache = {"x": x, "h": [h], "P": [], "Q": [], "a": [], "u": [], "pre": [], "s": s, "W": Wg}
    degc = np.maximum(g.deg, 1)[:, None].astype(np.float64)
    for l in range(NL):
        P = r(h @ Wg[f"W_p{l}"].T)
        Q = h @ Wg[f"W_q{l}"].T + Wg[f"b_m{l}"]
        pre = Q[g.src] + P[g.dst] + g.e @ Wg[f"C{l}"].T
        m = _relu(pre)
        asum = np.zeros((N, H))
        np.add.at(asum, g.src, m)
        a = r(np.where(g.deg[:, None] > 0, asum / degc, 0.0))
        u = np.concatenate([h, a], axis=1) @ Wg[f"W_u{l}"].T + Wg[f"b_u{l}"]
        hn = r(h + _relu(u))
        for k, val in (("P", P), ("Q", Q), ("a", a), ("u", u), ("pre", pre)):
            cache[k].append(val)
        cache["h"].append(hn)
        h = hn
    out = h @ Wg["W_d"].T + Wg["b_d"]
    z = v + act[:, None] * Wg["beta"][None, :] * out / s
    cache["out"] = out
    return z, out, cache


def loss_grad(w, g: Graph, v, t, ctx, act, emulate: bool = True):
    """Loss and the gradient of every trained parameter (flat, NPARAM; alpha/beta entries 0)."""
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    z, out, c = forward(w, g, v, ctx, act, emulate)
    Wg, s = c["W"], c["s"]
    N = v.shape[0]
    nm = max(5.0 * act.sum(), 1.0)
    rt = s * (t - v) / Wg["beta"][None, :]
    diff = out - rt
    loss = float((act[:, None] * diff * diff).sum() / nm)
    dout = 2.0 * act[:, None] * diff / nm
    gr = {n: np.zeros(sh) for n, (_, sh) in OFFSETS.items()}
    h3 = c["h"][NL]
    gr["W_d"] = dout.T @ h3
    gr["b_d"] = dout.sum(axis=0)
    dh = dout @ Wg["W_d"]
    degc = np.maximum(g.deg, 1)[:, None].astype(np.float64)
    for l in reversed(range(NL)):
        h, a, u, P, Q, pre = c["h"][l], c["a"][l], c["u"][l], c["P"][l], c["Q"][l], c["pre"][l]
        du = dh * (u > 0)
        dub = r(du)
        ha = np.concatenate([h, a], axis=1)
        gr[f"W_u{l}"] = dub.T @ ha
        gr[f"b_u{l}"] = du.sum(axis=0)
        dha = dub @ Wg[f"W_u{l}"]
        dh_prev = dh + dha[:, :H]
        dms = np.where(g.deg[:, None] > 0, dha[:, H:] / degc, 0.0)
        dpre = (pre > 0) * dms[g.src]
        dQ = np.zeros((N, H))
        np.add.at(dQ, g.src, dpre)
        dP = np.zeros((N, H))
        np.add.at(dP, g.dst, dpre)
        gr[f"C{l}"] = dpre.T @ g.e
        gr[f"b_m{l}"] = dQ.sum(axis=0)
        dQb, dPb = r(dQ), r(dP)
        gr[f"W_q{l}"] = dQb.T @ h
        gr[f"W_p{l}"] = dPb.T @ h
        dh = dh_prev + dQb @ Wg[f"W_q{l}"] + dPb @ Wg[f"W_p{l}"]
    h0 = c["h"][0]
    dpe = r(dh * (h0 > 0))
    gr["W_e"] = dpe.T @ c["x"]
    gr["b_e"] = (dh * (h0 > 0)).sum(axis=0)
    flat = np.zeros(NPARAM)
    for n, (o, sh) in OFFSETS.items():
        if n in ("alpha", "beta"):
            continue
        flat[o:o + int(np.prod(sh))] = gr[n].reshape(-1)
    return loss, flat, z
