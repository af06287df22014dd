"""Training and evaluation of the learned right preconditioner (flexible GMRES).

The preconditioner has no counterpart in the reference: PHASTA's matrix-free GMRES
(solmfg.f:221-340) is preconditioned by the 5x5 block-diagonal LU of i3lu.f alone.  Here a
message-passing network over the mesh edges maps a Krylov vector v of the block-diagonal
preconditioned operator A~ = L^-1 J U^-1 to z ~ A~^-1 v; ``precond = PHGPU_PRECOND_LEARNED``
makes the GMRES cycle flexible with z_j = P(v_j), and the block-diagonal method stays the
fallback (include/phgpu.h describes the policy).

Everything numerical runs on the GPU in libphgpu.so (csrc/learn.cu): the network's forward
and backward kernels (BF16 tensor-core GEMMs, FP32 accumulation), the Adam update and the
pair collection.  This module chooses the training states, drives the plain solver that
produces the pairs, and calls the training entry point.

Training pairs (v, t) come from block-diagonal solves of seeded perturbed states: w = U Dy is
the solve's Krylov-space solution, v = A~ w / ||A~ w||, t = w / ||A~ w|| (so A~ t = v exactly).
Pairs also come from the solve's Krylov basis vectors u_j (v = A~ u_j / ||A~ u_j||): the
network is applied to Krylov vectors inside flexible GMRES, not only to residuals, and without
them the trained network does not cut iterations.

Two state recipes (``PairRecipe.kind``):
  * "channel" (the learned-preconditioner workload's recipe): the channel mesh, uniform flow along
    x plus seeded Gaussian noise of sigma 0.5-5% of the free stream, Mach 0.1-0.6, half of the
    states with random-phase Fourier velocity modes on top; the inflow values follow the Mach
    number (phgpu_set_bc);
  * "periodic" (for the fully periodic decaying-vortex workload): a periodic [0, 2 pi]^3 box,
    thirds of Taylor-Green vortices, Fourier-mode fields and uniform flows in random directions,
    Mach 0.1-0.6, noise 0.1-5%, Re 1000-2000.
Each state gives the pairs of the three Newton iterations of one time step.  The network is
local (three edge hops) and its inputs are normalised, so pairs from a small mesh train the
operator of the large one.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import mesh

H, F_IN, NL, NOUT = 64, 48, 3, 5


def param_offsets() -> dict:
    """Offsets of the flat weight array (include/phgpu.h)."""
    lay = [("W_e", (H, F_IN)), ("b_e", (H,))]
    for l in range(NL):
        lay += [(f"W_p{l}", (H, H)), (f"W_q{l}", (H, H)), (f"b_m{l}", (H,)), (f"C{l}", (H, 3)),
                (f"W_u{l}", (H, 2 * H)), (f"b_u{l}", (H,))]
    lay += [("W_d", (NOUT, H)), ("b_d", (NOUT,)), ("alpha", (NOUT,)), ("beta", (NOUT,))]
    out, o = {}, 0
    for n, s in lay:
        out[n] = (o, s)
        o += int(np.prod(s))
    assert o == L.PHGPU_NET_NPARAM
    return out


def init_weights(seed: int = 1) -> np.ndarray:
    """He-scaled normal GEMM weights, zero biases and a zero decoder: the untrained network is the
    identity, i.e. flexible GMRES starts as the plain block-diagonal method."""
    g = np.random.default_rng(seed)
    w = np.zeros(L.PHGPU_NET_NPARAM, np.float32)
    for n, (o, s) in param_offsets().items():
        size = int(np.prod(s))
        if n.startswith("W_") and n != "W_d":
            scale = math.sqrt(2.0 / s[1]) * (0.5 if n.startswith("W_u") else 1.0)
            w[o:o + size] = (g.standard_normal(size) * scale).astype(np.float32)
        elif n.startswith("C"):
            w[o:o + size] = (0.5 * g.standard_normal(size)).astype(np.float32)
        elif n in ("alpha", "beta"):
            w[o:o + size] = 1.0
    return w


def channel_bc(case: mesh.Case, mach: float) -> np.ndarray:
    """BC(nshg, 6) of the channel's Dirichlet inflow for the free stream at ``mach``."""
    fs = mesh.freestream(mach)
    BC = np.array(case.BC, dtype=np.float64, copy=True)
    t = ((case.iBC >> 1) & 1) == 1
    v = ((case.iBC >> 3) & 7) == 7
    BC[1, t] = fs["T"]
    BC[2, v], BC[3, v], BC[4, v] = fs["u"], 0.0, 0.0
    return BC


@dataclass
class PairRecipe:
    kind: str = "channel"            # "channel" or "periodic"
    sigma: tuple = (0.005, 0.05)     # log-uniform noise level (fraction of the free stream)
    mach: tuple = (0.1, 0.6)         # uniform Mach number
    re: tuple = (1000.0, 1000.0)     # uniform Reynolds number
    fourier: float = 0.5             # share of states with Fourier velocity modes on top
    newton: int = 3                  # solves per state (Newton iterations of one time step)
    krylov: int = 8                  # pairs from Krylov vectors of each solve (besides its solution)


def training_mesh(n: int, recipe: PairRecipe | None = None):
    """The mesh the recipe's states live on: (case, physics dict)."""
    recipe = recipe or PairRecipe()
    return mesh.periodic_vortex_case(n) if recipe.kind == "periodic" else mesh.channel_case(n)


def state(case: mesh.Case, k: int, seed: int, recipe: PairRecipe):
    """Seeded training state k: (mach, re, y)."""
    g = np.random.default_rng([seed, k])
    mach = float(g.uniform(*recipe.mach))
    re = float(g.uniform(*recipe.re))
    sigma = float(math.exp(g.uniform(math.log(recipe.sigma[0]), math.log(recipe.sigma[1]))))
    if recipe.kind == "periodic":
        which = k % 3
        if which == 0:
            return mach, re, mesh.vortex_state(case, mach=mach, noise=sigma, seed=int(g.integers(1, 2 ** 31)))
        if which == 1:
            return mach, re, mesh.fourier_state(case, mach, kmax=4, noise=sigma, seed=int(g.integers(1, 2 ** 31)))
        y = mesh.uniform_state(case, mach, sigma=sigma, seed=int(g.integers(1, 2 ** 31))).reshape(5, -1).copy()
        d = g.standard_normal(3)
        d /= np.linalg.norm(d)
        y[:3] = y[0][None, :] * d[:, None] + y[1:3].sum(axis=0)[None, :] / 2.0
        return mach, re, mesh.apply_bc_state(case, y.reshape(-1))
    y = mesh.uniform_state(case, mach, sigma=sigma, seed=int(g.integers(1, 2 ** 31)))
    if g.uniform() < recipe.fourier:
        amp = float(g.uniform(0.1, 0.3))
        yf = mesh.fourier_state(case, mach, kmax=4, seed=int(g.integers(1, 2 ** 31)))
        y = y.reshape(5, -1).copy()
        y[:3] += amp * yf.reshape(5, -1)[:3]
        y = mesh.apply_bc_state(case, y.reshape(-1))
    return mach, re, y


def collect_pairs(g, case: mesh.Case, n_pairs: int, seed: int = 1, recipe: PairRecipe | None = None) -> dict:
    """Fill the context's training set with n_pairs pairs from block-diagonal solves (the GpuSolver
    ``g`` must be mixed precision with the linearized product on the recipe's mesh ``case``)."""
    recipe = recipe or PairRecipe()
    g.set_params(precond=L.PHGPU_PRECOND_BDIAG)
    g.net_pairs(n_pairs)
    slot, k, its = 0, 0, []
    t0 = time.perf_counter()
    while slot < n_pairs:
        mach, re, y0 = state(case, k, seed, recipe)
        dt = mesh.cfl_dt(case, mach)
        if recipe.kind == "channel":
            g.set_bc(channel_bc(case, mach))
        g.set_params(rmu=1.0 / re, istep=1, eGMRES=0.0, **mesh.time_params(0.5, dt))
        y, ac = y0, np.zeros_like(y0)
        ac0 = np.zeros_like(y0)
        for it in range(1, recipe.newton + 1):
            if slot >= n_pairs:
                break
            g.set_params(iter=it)
            _, _, Dy, st = g.SolMFG(y, ac)
            g.net_collect(slot)
            its.append(st.iKs)
            slot += 1
            for j in range(1, min(recipe.krylov, st.iKs) + 1):
                if slot >= n_pairs:
                    break
                g.net_collect(slot, j)
                slot += 1
            y, ac = g.itrCorrect(y, ac, y0, ac0, Dy)
        k += 1
    return {"pairs": n_pairs, "states": k, "krylov_iterations_mean": float(np.mean(its)),
            "seconds": time.perf_counter() - t0}


def train(g, case: mesh.Case, n_pairs: int = 2000, epochs: int = 8, lr: float = 1e-3, seed: int = 1,
          recipe: PairRecipe | None = None, weights: np.ndarray | None = None) -> tuple[np.ndarray, dict]:
    """Collect pairs and train on the GPU; returns (weights, report)."""
    rep = {"collect": collect_pairs(g, case, n_pairs, seed, recipe)}
    g.net_set_weights(init_weights(seed) if weights is None else weights)
    rep["train"] = g.net_train(epochs, lr=lr, seed=seed)
    return g.net_get_weights(), rep


WEIGHTS_DIR = __import__("pathlib").Path(__file__).resolve().parent / "weights"
DEFAULT_WEIGHTS = WEIGHTS_DIR / "precond_periodic16.f32"
# the command that made DEFAULT_WEIGHTS (on one GB300)
DEFAULT_RECIPE = dict(kind="periodic", n=16, pairs=2000, epochs=10, lr=1e-3, seed=3, krylov=8,
                      sigma=(0.001, 0.05), re=(1000.0, 2000.0))


def load_weights(path=None) -> np.ndarray:
    """A weight file written by ``python -m phasta_gb300.learn`` (PHGPU_NET_NPARAM float32 values)."""
    w = np.fromfile(str(path or DEFAULT_WEIGHTS), dtype="<f4")
    if w.size != L.PHGPU_NET_NPARAM:
        raise ValueError(f"{path}: {w.size} values, expected {L.PHGPU_NET_NPARAM}")
    return w


def train_default(out=None, **over) -> dict:
    """Train the default network (the periodic recipe on a 16^3 x 6 box) on the GPU and write it."""
    from .solver import GpuSolver, make_params
    cfg = dict(DEFAULT_RECIPE, **over)
    recipe = PairRecipe(kind=cfg["kind"], krylov=cfg["krylov"], sigma=tuple(cfg["sigma"]), re=tuple(cfg["re"]))
    case, ph = training_mesh(cfg["n"], recipe)
    p = make_params(ph["mu"], ph["dt"], Kspace=20, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                    outer_residual=L.PHGPU_RES_SPLITDF)
    g = GpuSolver(case, p)
    w, rep = train(g, case, n_pairs=cfg["pairs"], epochs=cfg["epochs"], lr=cfg["lr"], seed=cfg["seed"], recipe=recipe)
    g.close()
    out = __import__("pathlib").Path(out or DEFAULT_WEIGHTS)
    out.parent.mkdir(parents=True, exist_ok=True)
    w.astype("<f4").tofile(str(out))
    return {"recipe": cfg, **rep, "file": str(out)}


def probe(n: int, reps: int = 3, weights=None) -> dict:
    """Set the network up on the n^3 x 6 decaying-vortex mesh, run one mixed-precision Newton
    iteration (its features), then apply the network ``reps`` times and one linearized product
    (phgpu_sweep_dev 17 and 2): the timing probe the kernel profiles are taken on."""
    import time as _t
    from .solver import GpuSolver, make_params
    case, ph = mesh.periodic_vortex_case(n)
    p = make_params(ph["mu"], ph["dt"], Kspace=20, precision=L.PHGPU_MIXED, ap_mode=L.PHGPU_AP_LINEAR,
                    outer_residual=L.PHGPU_RES_SPLITDF, precond=L.PHGPU_PRECOND_LEARNED)
    g = GpuSolver(case, p)
    g.net_set_weights(load_weights(weights))
    y = mesh.vortex_state(case)
    g.upload(y, np.zeros_like(y), y, np.zeros_like(y))
    g.newton_dev()
    g.net_features()
    g.sweep_dev(5)
    t0 = _t.perf_counter()
    for _ in range(reps):
        g.sweep_dev(17)
    g.sweep_dev(2)
    g.download()
    out = {"n": n, "nodes": case.nshg, "edges": int(len(g.net_graph()[1])), "seconds": _t.perf_counter() - t0}
    g.close()
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train the learned preconditioner on the GPU and write its weights")
    ap.add_argument("--out", default=None)
    ap.add_argument("--kind", default=DEFAULT_RECIPE["kind"], choices=["periodic", "channel"])
    ap.add_argument("--n", type=int, default=DEFAULT_RECIPE["n"])
    ap.add_argument("--pairs", type=int, default=DEFAULT_RECIPE["pairs"])
    ap.add_argument("--epochs", type=int, default=DEFAULT_RECIPE["epochs"])
    ap.add_argument("--seed", type=int, default=DEFAULT_RECIPE["seed"])
    ap.add_argument("--probe", type=int, default=0, help="time the trained network on an N^3 x 6 vortex mesh instead")
    a = ap.parse_args()
    if a.probe:
        print(json.dumps(probe(a.probe)))
    else:
        print(json.dumps(train_default(a.out, kind=a.kind, n=a.n, pairs=a.pairs, epochs=a.epochs, seed=a.seed)))
