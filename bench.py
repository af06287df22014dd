"""Benchmark of the compressible Newton-Krylov hot path on one GB300.

Headline workload (the full-scale single-GPU case of the benchmark definitions):
a periodic [0, 2 pi]^3 cube of 192^3 hexes x 6 = 42,467,328 linear tets, 7,189,057
stored nodes (193^3, periodic slaves stored as in the reference), decaying vortex
u = U0 sin x cos y cos z, v = -U0 cos x sin y cos z, w = 0, Mach 0.1, Re 1600,
uniform p and T, seeded 0.1% noise; generalized alpha (rho_inf = 0.5) at CFL 1,
GMRES Kspace 20, tol 1e-3, 3 Newton iterations per time step.  Synthetic data
(no mesh files exist for it).

A "step" is one Newton iteration (one flow solve of the itrdrv multi-corrector:
SolMFG + itrCorrect + itrBC); steps run in time steps of 3 iterations.
``value`` = elements x steps / device time (CUDA events on the solver's stream),
inputs resident in HBM, for the learned-preconditioner mixed-precision form:
FP32 assembly and linearized products, the learned network (BF16 tensor-core
GEMMs) as the right preconditioner of flexible GMRES with the block-diagonal
fallback, FP64 outer residual, dots, Givens and LU.  Objects beside it:
``plain_mixed`` (the same precision, block-diagonal GMRES only), ``plain_fp64``
(the reference arithmetic on the same GPU: FP64 everywhere, finite-difference
Au1MFG, block-diagonal GMRES), both timed with CUDA events, with the speed-ups;
``channel`` (the 128^3 x 6 channel workload).
``e2e`` = the headline form through the host-buffer C ABI (phgpu_time_step) on
pinned host buffers, host<->device copies inside the timed region.  State and
mesh exceed the 129 MB L2, so no flush is needed between steps.

``--impl reference`` times the reference algorithm's CPU restatement (the
oracle) with all host threads on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NEWTON_PER_TIMESTEP = 3


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        # one nvidia-smi process streaming a sample every 50 ms (-lms), started before the timed region
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", "50"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        for line in self._proc.stdout:
            if self._stop.is_set():
                break
            line = line.strip()
            if line:
                self.samples.append([s.strip() for s in line.split(",")])

    def __enter__(self):
        self._proc = None
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.15)  # the sampling process is up before the timed region starts
        self.samples.clear()
        return self

    def __exit__(self, *a):
        time.sleep(0.06)
        self._stop.set()
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].strip() == "Active"})
        pw = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "power_w_max": max(pw) if pw else None, "samples": len(self.samples)}


def replica_throughput(local_ms: float, elements: int, steps: int, device: str = "cpu"):
    """Replicas only: every rank solves its own copy; the job time is the max over ranks and
    the job throughput is world * elements * steps / that time.  No data-path collective."""
    world = 1
    try:
        import torch.distributed as tdist
        if tdist.is_available() and tdist.is_initialized():
            import torch
            world = tdist.get_world_size()
            t = torch.tensor([local_ms], dtype=torch.float64, device=device)
            tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
            local_ms = float(t.item())
    except ImportError:
        pass
    return local_ms, world * elements * steps / (local_ms / 1e3)


WORKLOADS = {
    "vortex": "periodic decaying vortex {n}^3x6 tets Mach0.1 Re1600 +0.1% noise, Kspace20 tol1e-3, 3 Newton/step",
    "channel": "channel {n}^3x6 tets Mach0.3 Re1000, Kspace20 tol1e-3, 3 Newton/step",
    "layered": "connected periodic box {n}x{n}x(n + n/20 + 13n/20) cells of hexes, prisms and tets, Fourier modes "
               "k<=8 Mach 0.35, Kspace20 tol1e-3, 3 Newton/step",
}


def make_workload(n: int, precision: str, kind: str = "channel", precond: int = 0):
    from phasta_gb300 import _lib as L
    from phasta_gb300 import mesh
    from phasta_gb300.solver import make_params

    if kind == "vortex":
        case, ph = mesh.periodic_vortex_case(n, mach=0.1, re=1600.0)
        y0 = mesh.vortex_state(case, mach=0.1, noise=1e-3)
    elif kind == "layered":
        case, ph = mesh.layered_case(n, n, max(1, n // 20), max(1, (13 * n) // 20), mach=0.35)
        y0 = mesh.fourier_state(case, 0.35, kmax=8, noise=1e-3)
    else:
        case, ph = mesh.channel_case(n, mach=0.3, re=1000.0)
        y0 = mesh.uniform_state(case, 0.3, sigma=0.01)
    prec = L.PHGPU_MIXED if precision == "mixed" else L.PHGPU_FP64
    ap = L.PHGPU_AP_LINEAR if precision == "mixed" else L.PHGPU_AP_FD
    res = L.PHGPU_RES_SPLITDF if precision == "mixed" else L.PHGPU_RES_FP64
    params = make_params(ph["mu"], ph["dt"], rho_inf=0.5, Kspace=20, etol=1e-3, minIters=1,
                         precision=prec, ap_mode=ap, outer_residual=res,
                         precond=precond if precision == "mixed" else L.PHGPU_PRECOND_BDIAG)
    ac0 = np.zeros_like(y0)
    return case, params, y0, ac0


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_newton(g, case, y0, ac0, steps, stream, clock_dev=None, reset=None):
    """Time ``steps`` Newton iterations (time steps of 3) on resident data with CUDA events."""
    import torch

    def run_steps(k):
        done = 0
        while done < k:
            nitr = min(NEWTON_PER_TIMESTEP, k - done)
            g.time_step_dev(nitr)
            done += nitr

    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    if reset:
        reset()
    torch.cuda.synchronize()
    l0 = g.kernel_launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(clock_dev) if clock_dev is not None else None
    if clk:
        clk.__enter__()
    ev0.record(stream)
    t0 = time.perf_counter()
    run_steps(steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if clk:
        clk.__exit__()
    return {"ms": ev0.elapsed_time(ev1), "wall_s": wall, "launches": g.kernel_launches - l0,
            "clocks": clk.summary() if clk else None}


def convergence(g, y0, ac0, reset=None):
    """One time step's Newton iterations outside the timed region: Krylov iterations and the FP64
    nonlinear residual (unpreconditioned, after BCs) before each and after the last."""
    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    if reset:
        reset()
    r0 = g.residual_norm_dev()
    iks, rn, net = [], [], []
    for it in range(1, NEWTON_PER_TIMESTEP + 1):
        g.set_params(iter=it)
        st = g.newton_dev()
        iks.append(st.iKs)
        rn.append(st.rnorm)
        net.append({"net_its": st.net_its, "outcome": ["used", "fell_back", "plain"][st.net_fallback]})
    r_end = g.residual_norm_dev()
    return {"krylov_iterations": iks, "residual_before_each": rn, "rel_residual_after_3": r_end / r0,
            "learned": net}, g.download()[0]


def run_gpu(args, rank, world):
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300 import learn
    from phasta_gb300.solver import GpuSolver

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    kind, n = args.workload, args.n
    wl = WORKLOADS[kind].format(n=n)
    weights = learn.load_weights(args.weights)
    res = {}
    # ---- the headline: learned-preconditioner mixed-precision form ----
    case, params, y0, ac0 = make_workload(n, "mixed", kind, precond=L.PHGPU_PRECOND_LEARNED)
    E = case.nelem
    t_setup = time.perf_counter()
    g = GpuSolver(case, params)
    g.net_set_weights(weights)  # builds the edge graph
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.ExternalStream(g.stream())
    reset = lambda: g.net_set_weights(weights)  # noqa: E731  the fallback statistics start again
    g.upload(y0, ac0, y0, ac0)
    for _ in range(max(1, args.warmup // NEWTON_PER_TIMESTEP)):
        g.time_step_dev(NEWTON_PER_TIMESTEP)
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
    u0 = g.net_usage()
    t = run_newton(g, case, y0, ac0, args.steps, stream, clock_dev=dev, reset=reset)
    u1 = g.net_usage()
    ms, value = replica_throughput(t["ms"], E, args.steps, device="cuda")
    usage = {k: u1[k] - u0[k] for k in ("used", "fell_back", "plain")}
    usage["off_at_end"] = u1["off"]
    conv, y_learned = convergence(g, y0, ac0, reset=reset)

    # e2e: pinned host buffers through the reference-facing time-step call (phgpu_time_step:
    # H2D of yold/acold, 3 Newton iterations, D2H of y/ac/yold/acold, every time step)
    def pinned(a):
        tt = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        h = tt.numpy()
        h[:] = a
        return tt, h
    keep = [pinned(y0), pinned(ac0), pinned(y0), pinned(ac0)]
    yold, acold, y, ac = (k[1] for k in keep)
    g.set_params(istep=0, eGMRES=0.0)
    reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ksteps = max(1, args.steps // NEWTON_PER_TIMESTEP)
    for _ in range(ksteps):
        g.time_step_into(yold, acold, y, ac, NEWTON_PER_TIMESTEP)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_steps = ksteps * NEWTON_PER_TIMESTEP
    e2e = {"value": world * E * e2e_steps / e2e_s, "unit": "elements/s",
           "h2d_bytes_per_step": int(2 * 5 * case.nshg * 8 / NEWTON_PER_TIMESTEP),
           "d2h_bytes_per_step": int(4 * 5 * case.nshg * 8 / NEWTON_PER_TIMESTEP)}
    roof = kernel_roofline(g, case, stream, sum(conv["krylov_iterations"]) / NEWTON_PER_TIMESTEP)
    tuning = g.tuning()
    g.close()
    del g

    # ---- the same precision without the network (block-diagonal GMRES) ----
    case, params, y0, ac0 = make_workload(n, "mixed", kind, precond=L.PHGPU_PRECOND_BDIAG)
    gp = GpuSolver(case, params)
    sp = torch.cuda.ExternalStream(gp.stream())
    gp.upload(y0, ac0, y0, ac0)
    for _ in range(max(1, args.warmup // NEWTON_PER_TIMESTEP)):
        gp.time_step_dev(NEWTON_PER_TIMESTEP)
    tp = run_newton(gp, case, y0, ac0, args.steps, sp)
    conv_p, y_plain = convergence(gp, y0, ac0)
    gp.close()
    del gp
    plain_mixed = {"value": E * args.steps / (tp["ms"] / 1e3), "ms_per_step": tp["ms"] / args.steps, **conv_p,
                   "gpu_launches": tp["launches"]}

    result = {
        "metric": "Newton-step throughput to 1e-3 relative nonlinear residual, learned-FGMRES mixed precision "
                  "(elements/s)",
        "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 assembly/Ap; bf16 network GEMMs (f32 accumulate); double-float Galerkin flux; "
                 "f64 dots, Givens, LU",
        "data": "synthetic",
        "config": {"workload": wl, "elements": E, "nodes": case.nshg, "precision": "mixed",
                   "preconditioner": "learned (flexible GMRES, block-diagonal fallback)",
                   "weights": os.path.relpath(str(args.weights or learn.DEFAULT_WEIGHTS), str(ROOT)),
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "e2e": e2e, "gpu_launches": int(t["launches"]), "wall_s": t["wall_s"], "setup_s": t_setup,
        "newton": conv, "learned_usage": usage, "plain_mixed": plain_mixed,
        "speedup_vs_plain_mixed": plain_mixed["ms_per_step"] / (ms / args.steps),
        "roofline": roof, "clocks": t["clocks"],
        "sweep_tuning": {"lin_minb": tuning["lin_minb"], "ress_minb": tuning["ress_minb"], "how": tuning["how"],
                         "lin_ms": {str(k): v for k, v in tuning["lin_ms"].items()},
                         "ress_ms": {str(k): v for k, v in tuning["ress_ms"].items()}},
    }
    result["state_rel_diff_learned_vs_plain_mixed"] = float(np.linalg.norm(y_learned - y_plain) /
                                                            np.linalg.norm(y_plain))
    if not args.skip_fp64:
        result["plain_fp64"], y64 = fp64_plain(args, kind, n)
        result["plain_fp64"]["state_rel_diff_vs_learned"] = float(np.linalg.norm(y_learned - y64) / np.linalg.norm(y64))
        result["speedup_vs_plain_fp64"] = result["plain_fp64"]["ms_per_step"] / (ms / args.steps)
    if not args.skip_channel:
        result["channel"] = channel_object(args, weights)
    if not args.skip_mixed:
        result["mixed_topology"] = mixed_topology_object(args)
    if not args.skip_order:
        result["node_order"] = node_order_object(args)
    if not args.skip_sparse:
        result["sparse_solver"] = sparse_solver(args)
        result["ebe_solver"] = sparse_solver(args, ebe=True)
    return result


def launch_list_steps(args):
    """Two time steps of the block-diagonal mixed-precision form, launched kernel by kernel (config
    no_graph = 1: the same kernels as the step graph) after one time step of warm-up."""
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300 import build
    from phasta_gb300.solver import GpuSolver
    build.build()
    case, params, y0, ac0 = make_workload(args.n, "mixed", args.workload, precond=L.PHGPU_PRECOND_BDIAG)
    g = GpuSolver(case, dict(params, no_graph=1))
    g.upload(y0, ac0, y0, ac0)
    g.time_step_dev(NEWTON_PER_TIMESTEP)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    iks = []
    for _ in range(2):
        iks.append(g.time_step_dev(NEWTON_PER_TIMESTEP).iKs)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / (2 * NEWTON_PER_TIMESTEP) * 1e3
    out = {"workload": WORKLOADS[args.workload].format(n=args.n), "ms_per_newton_wall": ms, "last_iKs": iks,
           "tuning": {k: v for k, v in g.tuning().items() if k in ("lin_minb", "ress_minb", "how")}}
    g.close()
    return out


def mixed_topology_object(args):
    """The mixed-topology workload: one connected periodic box of 80 x 80 cells in x, y whose z
    layers are 80 of hexes (512,000), 4 of prisms (51,200) and 52 of Kuhn tets (1,996,800),
    sharing their interface nodes; random-phase Fourier velocity modes (k <= 8) at Mach 0.35 with
    0.1% noise; mixed precision, block-diagonal GMRES, 10 time steps x 3 Newton iterations."""
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300 import mesh
    from phasta_gb300.solver import GpuSolver, make_params
    n = args.mixed_n
    lay = (n, max(1, n // 20), max(1, (13 * n) // 20))
    case, ph = mesh.layered_case(n, *lay, mach=0.35)
    p = make_params(ph["mu"], ph["dt"], rho_inf=0.5, Kspace=20, etol=1e-3, precision=L.PHGPU_MIXED,
                    ap_mode=L.PHGPU_AP_LINEAR, outer_residual=L.PHGPU_RES_SPLITDF)
    y0 = mesh.fourier_state(case, 0.35, kmax=8, noise=1e-3)
    ac0 = np.zeros_like(y0)
    g = GpuSolver(case, p)
    s = torch.cuda.ExternalStream(g.stream())
    g.upload(y0, ac0, y0, ac0)
    g.time_step_dev(NEWTON_PER_TIMESTEP)
    steps = 10 * NEWTON_PER_TIMESTEP
    t = run_newton(g, case, y0, ac0, steps, s)
    conv, _ = convergence(g, y0, ac0)
    E = case.nelem + case.nhex + case.nwedge
    g.close()
    return {"workload": f"connected periodic box {n}x{n}x{sum(lay)} cells: {case.nhex} hexes, {case.nwedge} prisms, "
                        f"{case.nelem} tets sharing interface nodes; Fourier modes k<=8 Mach 0.35; 10 time steps x 3 "
                        f"Newton", "elements": E, "nodes": case.nshg, "value": E * steps / (t["ms"] / 1e3),
            "unit": "elements/s", "ms_per_step": t["ms"] / steps, "gpu_launches": t["launches"], **conv,
            "launch": "tets: persistent pipelined kernel per colour; hexes and prisms: one launch per colour"}


def node_order_object(args):
    """The channel at --order-n^3 x 6 (mixed precision, block-diagonal GMRES) with its nodes in
    generation order, shuffled at random, and shuffled then renumbered by reverse Cuthill-McKee
    (phgpu_rcm_order): ms per Newton iteration over 2 time steps x 3 Newton iterations each."""
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300 import mesh
    from phasta_gb300.solver import GpuSolver, rcm_order
    n = args.order_n
    case, params, y0, ac0 = make_workload(n, "mixed", "channel", precond=L.PHGPU_PRECOND_BDIAG)
    shuf = np.random.default_rng(20261204).permutation(case.nshg)
    sh = mesh.renumber(case, shuf)
    t0 = time.perf_counter()
    perm, bw_shuf, bw_rcm = rcm_order(sh)
    t_rcm = time.perf_counter() - t0
    _, bw_gen, _ = rcm_order(case)
    ys, acs = mesh.renumber_field(y0, shuf, 5), mesh.renumber_field(ac0, shuf, 5)
    out = {"workload": WORKLOADS["channel"].format(n=n), "rcm_host_s": t_rcm}
    for name, m, y, ac, bw in (("generated", case, y0, ac0, bw_gen), ("shuffled", sh, ys, acs, bw_shuf),
                               ("rcm_of_shuffled", mesh.renumber(sh, perm), mesh.renumber_field(ys, perm, 5),
                                mesh.renumber_field(acs, perm, 5), bw_rcm)):
        g = GpuSolver(m, params)
        s = torch.cuda.ExternalStream(g.stream())
        g.upload(y, ac, y, ac)
        g.time_step_dev(NEWTON_PER_TIMESTEP)
        steps = 2 * NEWTON_PER_TIMESTEP
        t = run_newton(g, m, y, ac, steps, s)
        out[name] = {"ms_per_step": t["ms"] / steps, "bandwidth": int(bw)}
        g.close()
    return out


def channel_object(args, weights):
    """The 128^3 x 6 channel workload: block-diagonal and learned mixed-precision forms."""
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300.solver import GpuSolver
    out = {"workload": WORKLOADS["channel"].format(n=args.channel_n)}
    for name, pc in (("plain_mixed", L.PHGPU_PRECOND_BDIAG), ("learned", L.PHGPU_PRECOND_LEARNED)):
        case, params, y0, ac0 = make_workload(args.channel_n, "mixed", "channel", precond=pc)
        g = GpuSolver(case, params)
        reset = None
        if pc == L.PHGPU_PRECOND_LEARNED:
            g.net_set_weights(weights)
            reset = lambda g=g: g.net_set_weights(weights)  # noqa: E731
        s = torch.cuda.ExternalStream(g.stream())
        g.upload(y0, ac0, y0, ac0)
        g.time_step_dev(NEWTON_PER_TIMESTEP)
        steps = 2 * NEWTON_PER_TIMESTEP
        t = run_newton(g, case, y0, ac0, steps, s, reset=reset)
        conv, _ = convergence(g, y0, ac0, reset=reset)
        out[name] = {"value": case.nelem * steps / (t["ms"] / 1e3), "ms_per_step": t["ms"] / steps, **conv}
        if pc == L.PHGPU_PRECOND_LEARNED:
            out[name]["usage"] = g.net_usage()
        g.close()
    return out


def _time_sweep(g, stream, which, reps=10):
    import torch
    for _ in range(3):
        g.sweep_dev(which)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        g.sweep_dev(which)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps / 1e3


# The element sweeps of one mixed-precision Newton iteration and their compulsory
# HBM bytes (int4 connectivity per element; per node what the sweep must read and write):
#   ress: outer residual, reads y, ac (f64) and x (f64), writes res (f64)
#   full: FP32 block diagonal (BDiag-only variant), reads y, x (f32), writes BDiag (25 f32)
#   lin:  FP32 linearized product, reads the direction, base state, x (f32), reads and writes the product
SWEEPS = {
    "ress": (7, "k_chunk_ress_pipe (double-float constant flux + FP32 increment residual, cp.async-pipelined)",
             lambda E, N: 16 * E + N * (40 + 40 + 24 + 40)),
    "full": (3, "k_chunk_full<float, true> (FP32 block diagonal)", lambda E, N: 16 * E + N * (20 + 12 + 100)),
    "lin": (2, "k_chunk_lin_pipe (FP32 linearized Ap sweep, cp.async-pipelined)",
            lambda E, N: 16 * E + N * (20 + 20 + 12 + 40)),
}
# One application of the learned preconditioner (4 kernels): per node the direction (20 B) and
# context features (64 B) read, h and P (bf16, 128 B each) written by the encoder; per layer the
# CSR (4 B per edge), h read and written, P read (once, compulsory) and the next P written; the
# last layer reads v and writes z (20 B each) instead of writing h and P.
# encoder 340 B per node; two middle layers 512 B per node; the last layer 296 B per node (reads h, P, v,
# writes z); 4 B per edge of the CSR in each of the three layers
NET_BYTES = lambda N, nnz: N * (340 + 2 * 512 + 296) + 3 * 4 * nnz  # noqa: E731
# tensor-core flops per node of one application: encoder 48x64, per layer Q (64x64), update
# (128x64) and the next projection (64x64, two layers) or decoder (64x8)
NET_FLOPS = lambda N: N * 2 * (48 * 64 + 64 * 64 + 3 * (64 * 64 + 128 * 64) + 2 * 64 * 64 + 64 * 8)  # noqa: E731


def kernel_roofline(g, case, stream, krylov_per_newton):
    """Time each element sweep and the network alone; the roofline object is the one with the largest
    share of a Newton iteration."""
    g.sweep_dev(5)  # FP32 copies of the state
    g.sweep_dev(8)  # hi/lo copies for the split residual
    E, N = case.nelem, case.nshg
    peak, src = peaks()
    calls = {"ress": 1.0, "full": 1.0, "lin": krylov_per_newton}
    kernels = {}
    for key, (which, name, algo_f) in SWEEPS.items():
        t = _time_sweep(g, stream, which)
        algo = algo_f(E, N)
        kernels[key] = {"kernel": name, "ms": t * 1e3, "calls_per_newton": calls[key],
                        "ms_per_newton": t * 1e3 * calls[key], "algorithmic_bytes": algo,
                        "achieved_gbs": algo / t / 1e9, "elements_per_s": E / t}
    kernels["lin"]["per_chunk_kernel_ms"] = _time_sweep(g, stream, 15) * 1e3
    kernels["ress"]["per_chunk_kernel_ms"] = _time_sweep(g, stream, 16) * 1e3
    # the learned preconditioner (one application: encoder + 3 message-passing layers)
    try:
        g.net_features()
        t = _time_sweep(g, stream, 17)
        nnz = len(g.net_graph()[1])
        kernels["net"] = {"kernel": "k_net_enc + 3 x k_net_mp (learned preconditioner, mma.sync bf16)",
                          "ms": t * 1e3, "algorithmic_bytes": NET_BYTES(N, nnz), "achieved_gbs": NET_BYTES(N, nnz) / t / 1e9,
                          "tensor_tflops": NET_FLOPS(N) / t / 1e12, "edges": nnz,
                          "ms_vs_lin": t * 1e3 / kernels["lin"]["ms"]}
        kernels["net_features"] = {"ms": _time_sweep(g, stream, 18) * 1e3}
    except Exception as e:  # noqa: BLE001
        kernels["net"] = {"error": str(e)}
    # the reference formulation's exact flops per tet (the oracle's counting scalar): the work each
    # sweep stands for, per second
    fp = ROOT / "profiles" / "flops_per_element.json"
    if fp.exists():
        doc = json.loads(fp.read_text())
        peak32 = 152 * 128 * 2 * 2.070e9 / 1e12
        for key, path in doc["sweeps"].items():
            topo, mode = path.split(".")
            f = doc["per_element"][topo][mode]
            eff = f * E / (kernels[key]["ms"] / 1e3) / 1e12
            kernels[key]["reference_flops_per_element"] = f
            kernels[key]["reference_work_tflops"] = eff
            kernels[key]["reference_work_frac_of_fp32_peak"] = eff / peak32
    dom = max((k for k in SWEEPS), key=lambda k: kernels[k]["ms_per_newton"])
    k = kernels[dom]
    traffic, fp32 = None, None
    tp = ROOT / "profiles" / "sweep_traffic.json"
    if tp.exists():
        d = json.loads(tp.read_text())
        if dom in d:
            traffic = d[dom]["dram_bytes_per_element"] * E
            f = d[dom].get("fp32_flops_per_element")
            if f:
                peak32 = 152 * 128 * 2 * 2.070e9 / 1e12
                ach = f * E / (k["ms"] / 1e3) / 1e12
                fp32 = {"flops_per_element": f, "achieved_tflops": ach, "peak_tflops": peak32,
                        "frac": ach / peak32, "peak_source": "nominal FP32 CUDA-core peak",
                        "flops_source": "executed FP32 instructions (ncu) of the GPU's formulation",
                        "reference_flops_per_element": k.get("reference_flops_per_element"),
                        "reference_work_frac": k.get("reference_work_frac_of_fp32_peak")}
    return {"kernel": k["kernel"], "bound": "hbm", "achieved": k["achieved_gbs"], "peak": peak, "unit": "GB/s",
            "frac": k["achieved_gbs"] / peak, "peak_source": f"{src} hbm_gbs", "traffic": traffic,
            "algorithmic_bytes": k["algorithmic_bytes"], "launch_ms": k["ms"], "fp32": fp32, "sweeps": kernels}


def sparse_solver(args, ebe: bool = False):
    """The reference's sparse solver (SolGMRs on the assembled tangent) or, with ebe, its
    element-by-element solver (SolGMRe on stored element tangents) on the channel workload: FP32
    tangent and Krylov vectors."""
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300.solver import GpuSolver

    case, params, y0, ac0 = make_workload(args.channel_n, "mixed", "channel")
    params = dict(params, ap_mode=L.PHGPU_AP_EBE if ebe else L.PHGPU_AP_SPARSE)
    g = GpuSolver(case, params)
    stream = torch.cuda.ExternalStream(g.stream())
    g.upload(y0, ac0, y0, ac0)
    g.time_step_dev(NEWTON_PER_TIMESTEP)  # warm-up (builds the block structure)
    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    torch.cuda.synchronize()
    r0 = g.residual_norm_dev()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    iks = []
    for it in range(1, NEWTON_PER_TIMESTEP + 1):
        g.set_params(iter=it)
        iks.append(g.newton_dev().iKs)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / NEWTON_PER_TIMESTEP
    r_end = g.residual_norm_dev()
    E, N = case.nelem, case.nshg
    vb = 4
    if ebe:
        nnzb = 16 * E
        tan, spmv = 13, 14
        tan_bytes = 25 * vb * nnzb + N * 8 * vb + E * 16
        spmv_bytes = 25 * vb * nnzb + E * 16 + 2 * 5 * vb * N
    else:
        nnzb = g.nnz_tot
        tan, spmv = 9, 10
        tan_bytes = 25 * vb * nnzb + N * 8 * vb + E * (16 + 64)
        spmv_bytes = nnzb * (25 * vb + 4) + 4 * (N + 1) + 2 * 5 * vb * N
    t_tan = _time_sweep(g, stream, tan, reps=3)
    t_spmv = _time_sweep(g, stream, spmv, reps=10)
    g.close()
    return {"workload": WORKLOADS["channel"].format(n=args.channel_n), "ms_per_newton": ms,
            "value": E / ms * 1e3, "krylov_iterations": iks, "rel_residual_after_3": r_end / r0,
            "nnz_blocks": nnzb,
            "tangent": {"ms": t_tan * 1e3, "algorithmic_bytes": tan_bytes, "achieved_gbs": tan_bytes / t_tan / 1e9},
            "spmv": {"ms": t_spmv * 1e3, "algorithmic_bytes": spmv_bytes,
                     "achieved_gbs": spmv_bytes / t_spmv / 1e9}}


def fp64_plain(args, kind, n):
    """The reference arithmetic on the same GPU: FP64 everywhere, finite-difference Au1MFG,
    block-diagonal GMRES; one time step (3 Newton iterations) timed with CUDA events."""
    import torch

    from phasta_gb300.solver import GpuSolver

    case, params, y0, ac0 = make_workload(n, "fp64", kind)
    g = GpuSolver(case, params)
    stream = torch.cuda.ExternalStream(g.stream())
    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    torch.cuda.synchronize()
    r0 = g.residual_norm_dev()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    iks = []
    for it in range(1, NEWTON_PER_TIMESTEP + 1):
        g.set_params(iter=it)
        iks.append(g.newton_dev().iKs)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / NEWTON_PER_TIMESTEP
    r_end = g.residual_norm_dev()
    y = g.download()[0]
    g.close()
    return {"ms_per_step": ms, "value": case.nelem / ms * 1e3, "krylov_iterations": iks,
            "rel_residual_after_3": r_end / r0, "timing": "CUDA events, one time step"}, y


def cpu_sample(n_sample: int, kind: str = "vortex", steps: int = 1):
    """The oracle (reference algorithm, FP64, finite-difference Au1MFG) on host threads."""
    from oracle.pyoracle import Oracle

    case, params, y0, ac0 = make_workload(n_sample, "fp64", kind)
    threads = os.cpu_count() or 1
    o = Oracle(case, params, nthreads=threads, grouped=True)
    t0 = time.perf_counter()
    y, ac = y0, ac0
    for it in range(1, steps + 1):
        o.set_params(iter=it)
        y, ac, st, _ = o.newton(y, ac, y0, ac0)
    dt = time.perf_counter() - t0
    return {"value": case.nelem * steps / dt, "unit": "elements/s", "cores": threads, "kind": "port",
            "sample": f"{steps} Newton iteration(s) of the {kind} workload at {n_sample}^3x6 = {case.nelem} tets "
                      f"(FP64, Kspace 20, tol 1e-3, block-diagonal GMRES), {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return None
    n_s = args.cpu_sample_n
    vals = []
    for _ in range(args.warmup):
        cpu_sample(n_s, args.workload, steps=1)
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_sample(n_s, args.workload, steps=1)
        vals.append(last["value"])
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    return {"impl": "reference",
            "metric": "Newton-step throughput to 1e-3 relative nonlinear residual, learned-FGMRES mixed precision "
                      "(elements/s)",
            "value": v, "unit": "elements/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload].format(n=args.n), "sample_n": n_s,
                       "sample": f"1 Newton iteration of the same workload at {n_s}^3x6 per step"},
            "cpu_baseline": {**last, "value": v},
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60, help="Newton iterations timed (20 time steps x 3)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="vortex", choices=["vortex", "channel", "layered"])
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--channel-n", type=int, default=128)
    ap.add_argument("--weights", default=None, help="learned preconditioner weights (default: the committed file)")
    ap.add_argument("--cpu-sample-n", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-channel", action="store_true")
    ap.add_argument("--skip-mixed", action="store_true")
    ap.add_argument("--skip-order", action="store_true", help="leave out the node-order (RCM) object")
    ap.add_argument("--order-n", type=int, default=96)
    ap.add_argument("--mixed-n", type=int, default=80)
    ap.add_argument("--skip-sparse", action="store_true", help="leave out the assembled-tangent solver lines")
    ap.add_argument("--launch-list", action="store_true",
                    help="only run 2 time steps (after one of warm-up) of the block-diagonal mixed form of --workload "
                         "at --n, kernel by kernel (for an ncu launch list: kernels inside captured graphs are not "
                         "listed), and print ms per Newton iteration")
    args = ap.parse_args()
    rank, world, _ = _dist()
    if args.launch_list:
        print(json.dumps(launch_list_steps(args)))
        return
    if args.impl == "reference":
        out = run_reference(args)
        if out is not None:
            print(json.dumps(out))
        return
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    from phasta_gb300 import build
    if rank == 0:
        build.build()
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
    res = run_gpu(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_sample(args.cpu_sample_n, args.workload, steps=1)
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
