"""Benchmark of the compressible Newton-Krylov hot path on one GB300.

Workload (the at-scale case of the benchmark definitions): unit cube,
128^3 hexes x 6 = 12,582,912 linear tets, 2,146,689 stored nodes, periodic in
y and z, Dirichlet inflow / natural outflow in x, Mach 0.3, Re 1000, gamma 1.4,
Pr 0.72, uniform flow + seeded 1% Gaussian noise, generalized alpha
(rho_inf = 0.5) at CFL 1, GMRES Kspace 20, tol 1e-3, 3 Newton iterations per
time step.  Synthetic data (no mesh files exist for it).

A "step" is one Newton iteration (one flow solve of the itrdrv multi-corrector:
SolMFG + itrCorrect + itrBC).  Steps run in time steps of 3 iterations.
``value`` = elements x steps / device time, inputs resident in HBM;
``e2e`` = the same through the host-buffer C ABI (phgpu_time_step) on pinned host
buffers, host<->device copies inside the timed region.  The state and mesh (> 300 MB) exceed the
129 MB L2, so no flush is needed between steps.

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


def make_workload(n: int, precision: str):
    from phasta_gb300 import _lib as L
    from phasta_gb300 import mesh
    from phasta_gb300.solver import make_params

    case, ph = mesh.channel_case(n, mach=0.3, re=1000.0)
    prec = L.PHGPU_MIXED if precision == "mixed" else L.PHGPU_FP64
    ap = L.PHGPU_AP_LINEAR if precision == "mixed" else L.PHGPU_AP_FD
    res = L.PHGPU_RES_SPLITDF if precision == "mixed" else L.PHGPU_RES_FP64
    params = make_params(ph["mu"], ph["dt"], rho_inf=0.5, Kspace=20, etol=1e-3, minIters=1,
                         precision=prec, ap_mode=ap, outer_residual=res)
    y0 = mesh.uniform_state(case, 0.3, sigma=0.01)
    ac0 = np.zeros_like(y0)
    return case, params, y0, ac0


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_gpu(args, rank, world):
    import torch

    from phasta_gb300.solver import GpuSolver

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    case, params, y0, ac0 = make_workload(args.n, args.precision)
    E = case.nelem
    g = GpuSolver(case, params)
    stream = torch.cuda.ExternalStream(g.stream())

    def run_steps(k):
        done = 0
        while done < k:
            nitr = min(NEWTON_PER_TIMESTEP, k - done)
            g.time_step_dev(nitr)
            done += nitr

    g.upload(y0, ac0, y0, ac0)
    run_steps(args.warmup)
    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.barrier()
    torch.cuda.synchronize()
    l0 = g.kernel_launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        t0 = time.perf_counter()
        run_steps(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = g.kernel_launches - l0
    ms, value = replica_throughput(ev0.elapsed_time(ev1), E, args.steps, device="cuda")
    ms_per_step = ms / args.steps

    # convergence record of one time step (outside the timed region)
    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    r0 = g.residual_norm_dev()
    iks, rn = [], []
    for it in range(1, NEWTON_PER_TIMESTEP + 1):
        g.set_params(iter=it)
        st = g.newton_dev()
        iks.append(st.iKs)
        rn.append(st.rnorm)
    r_end = g.residual_norm_dev()
    y_mixed = g.download()[0]

    # e2e: pinned host buffers through the reference-facing time-step call (phgpu_time_step:
    # H2D of yold/acold, 3 Newton iterations, D2H of y/ac/yold/acold, every time step)
    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        h = t.numpy()
        h[:] = a
        return t, h
    keep = [pinned(y0), pinned(ac0), pinned(y0), pinned(ac0)]
    yold, acold, y, ac = (k[1] for k in keep)
    g.set_params(istep=0, eGMRES=0.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ksteps = max(1, args.steps // NEWTON_PER_TIMESTEP)
    for _ in range(ksteps):
        st = g.time_step_into(yold, acold, y, ac, NEWTON_PER_TIMESTEP)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_steps = ksteps * NEWTON_PER_TIMESTEP
    e2e = {"value": world * E * e2e_steps / e2e_s, "unit": "elements/s",
           "h2d_bytes_per_step": int(2 * 5 * case.nshg * 8 / NEWTON_PER_TIMESTEP),
           "d2h_bytes_per_step": int(4 * 5 * case.nshg * 8 / NEWTON_PER_TIMESTEP)}

    # the element sweep with the largest share of a Newton iteration
    roof = kernel_roofline(g, case, stream, args, sum(iks) / len(iks))
    result = {
        "metric": "Newton-step throughput to 1e-3 relative nonlinear residual (elements/s)",
        "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f32 assembly/Ap/stabilization; double-float Galerkin flux; f64 dots, Givens, LU"
                  if args.precision == "mixed" else "f64"),
        "data": "synthetic",
        "config": {"workload": f"channel {args.n}^3x6 tets Mach0.3 Re1000, Kspace20 tol1e-3, 3 Newton/step",
                   "elements": E, "nodes": case.nshg, "precision": args.precision,
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "e2e": e2e, "gpu_launches": int(launches), "wall_s": wall,
        "newton": {"krylov_iterations": iks, "residual_before_each": rn, "rel_residual_after_3": r_end / r0},
        "roofline": roof, "clocks": clk.summary(),
    }
    if args.precision == "mixed" and not args.skip_fp64:
        result["fp64_plain"], y64 = fp64_plain(args, case)
        # the error of the mixed-precision iterations against the FP64 ones, same start
        result["fp64_plain"]["state_rel_diff_vs_mixed"] = float(np.linalg.norm(y_mixed - y64) / np.linalg.norm(y64))
    if not args.skip_sparse:
        result["sparse_solver"] = sparse_solver(args)
        if args.precision == "mixed":
            result["ebe_solver"] = sparse_solver(args, ebe=True)
    g.close()
    return result


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


def kernel_roofline(g, case, stream, args, krylov_per_newton):
    """Time each element sweep alone; the roofline object is the one with the largest share of a Newton iteration."""
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
    # the linearized product with one CTA per chunk, for comparison with the pipelined kernel
    kernels["lin"]["per_chunk_kernel_ms"] = _time_sweep(g, stream, 15) * 1e3
    kernels["ress"]["per_chunk_kernel_ms"] = _time_sweep(g, stream, 16) * 1e3
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_newton"])
    k = kernels[dom]
    traffic, fp32 = None, None
    tp = ROOT / "profiles" / "sweep_traffic.json"
    if tp.exists():
        d = json.loads(tp.read_text())
        if dom in d:
            traffic = d[dom]["dram_bytes_per_element"] * E
            # the sweeps are FP32-issue bound: their executed FP32 flops (ncu instruction counts of
            # one colour launch, per element) against the CUDA-core peak of 152 SMs x 128 lanes
            # x 2 flops at 2070 MHz (nominal: the measured peaks cover HBM and tensor cores only)
            f = d[dom].get("fp32_flops_per_element")
            if f:
                peak32 = 152 * 128 * 2 * 2.070e9 / 1e12
                ach = f * E / (k["ms"] / 1e3) / 1e12
                fp32 = {"flops_per_element": f, "achieved_tflops": ach, "peak_tflops": peak32,
                        "frac": ach / peak32, "peak_source": "nominal FP32 CUDA-core peak"}
    return {"kernel": k["kernel"], "bound": "hbm", "achieved": k["achieved_gbs"], "peak": peak, "unit": "GB/s",
            "frac": k["achieved_gbs"] / peak, "peak_source": f"{src} hbm_gbs", "traffic": traffic,
            "algorithmic_bytes": k["algorithmic_bytes"], "launch_ms": k["ms"], "fp32": fp32, "sweeps": kernels}


def sparse_solver(args, ebe: bool = False):
    """The reference's sparse solver (SolGMRs on the assembled tangent) or, with ebe, its
    element-by-element solver (SolGMRe on stored element tangents) on the same workload: FP32
    tangent and Krylov vectors in mixed precision, FP64 throughout otherwise."""
    import torch

    from phasta_gb300 import _lib as L
    from phasta_gb300.solver import GpuSolver

    case, params, y0, ac0 = make_workload(args.n, args.precision)
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
    vb = 4 if args.precision == "mixed" else 8
    if ebe:
        if args.precision != "mixed":
            raise SystemExit("the element-by-element timing sweeps are FP32")
        nnzb = 16 * E
        tan, spmv = 13, 14
        # element storage written once; the product reads it, the connectivity and the vector
        tan_bytes = 25 * vb * nnzb + N * 8 * vb + E * 16
        spmv_bytes = 25 * vb * nnzb + E * 16 + 2 * 5 * vb * N
    else:
        nnzb = g.nnz_tot
        tan, spmv = (9, 10) if args.precision == "mixed" else (11, 12)
        # compulsory bytes: the tangent writes lhsK once and reads x, y, connectivity and block
        # maps; the product reads lhsK, its column list and the vector once and writes the result
        tan_bytes = 25 * vb * nnzb + N * 8 * vb + E * (16 + 64)
        spmv_bytes = nnzb * (25 * vb + 4) + 4 * (N + 1) + 2 * 5 * vb * N
    t_tan = _time_sweep(g, stream, tan, reps=3)
    t_spmv = _time_sweep(g, stream, spmv, reps=10)
    g.close()
    return {"ms_per_newton": ms, "value": E / ms * 1e3, "krylov_iterations": iks,
            "rel_residual_after_3": r_end / r0, "nnz_blocks": nnzb,
            "tangent": {"ms": t_tan * 1e3, "algorithmic_bytes": tan_bytes, "achieved_gbs": tan_bytes / t_tan / 1e9},
            "spmv": {"ms": t_spmv * 1e3, "algorithmic_bytes": spmv_bytes,
                     "achieved_gbs": spmv_bytes / t_spmv / 1e9}}


def fp64_plain(args, case):
    """The reference arithmetic on the same GPU: FP64 everywhere, finite-difference Au1MFG."""
    import torch

    from phasta_gb300.solver import GpuSolver

    case, params, y0, ac0 = make_workload(args.n, "fp64")
    g = GpuSolver(case, params)
    g.upload(y0, ac0, y0, ac0)
    g.set_params(istep=0, eGMRES=0.0)
    torch.cuda.synchronize()
    r0 = g.residual_norm_dev()
    t0 = time.perf_counter()
    iks = []
    for it in range(1, NEWTON_PER_TIMESTEP + 1):
        g.set_params(iter=it)
        st = g.newton_dev()
        iks.append(st.iKs)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    r_end = g.residual_norm_dev()
    y = g.download()[0]
    g.close()
    return {"ms_per_step": dt * 1e3 / NEWTON_PER_TIMESTEP,
            "value": case.nelem * NEWTON_PER_TIMESTEP / dt, "krylov_iterations": iks,
            "rel_residual_after_3": r_end / r0}, y


def cpu_sample(n_sample: int, steps: int = 1):
    """The oracle (reference algorithm, FP64, finite-difference Au1MFG) on host threads."""
    from oracle.pyoracle import Oracle

    case, params, y0, ac0 = make_workload(n_sample, "fp64")
    threads = os.cpu_count() or 1
    o = Oracle(case, params, nthreads=threads, grouped=True)
    t0 = time.perf_counter()
    y, ac = y0, ac0
    for it in range(1, steps + 1):
        o.set_params(iter=it)
        y, ac, st, _ = o.newton(y, ac, y0, ac0)
    dt = time.perf_counter() - t0
    return {"value": case.nelem * steps / dt, "unit": "elements/s", "cores": threads, "kind": "port",
            "sample": f"{steps} Newton iteration(s) of the channel case at {n_sample}^3x6 = {case.nelem} tets "
                      f"(FP64, Kspace 20, tol 1e-3), {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return None
    n_s = args.cpu_sample_n
    vals = []
    for _ in range(args.warmup):
        cpu_sample(n_s, steps=1)
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_sample(n_s, steps=2)
        vals.append(last["value"])
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    return {"impl": "reference", "metric": "Newton-step throughput to 1e-3 relative nonlinear residual (elements/s)",
            "value": v, "unit": "elements/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"channel {args.n}^3x6 tets Mach0.3 Re1000, Kspace20 tol1e-3, 3 Newton/step",
                       "sample_n": n_s},
            "cpu_baseline": {**last, "value": v},
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-sample-n", type=int, default=96)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-sparse", action="store_true", help="leave out the assembled-tangent solver line")
    args = ap.parse_args()
    rank, world, _ = _dist()
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
            res["cpu_baseline"] = cpu_sample(args.cpu_sample_n, steps=2)
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
