"""Benchmark of the GB300 elliptic solve (Poisson DOFs/s and time-to-tolerance).

One "step" is one complete ellipticSolve of the workload's Kershaw-box Poisson
problem to its relative tolerance, starting from the seeded right-hand side
already resident in HBM (`value`); `e2e` is the same solve through the
host-buffer C ABI call (nrsg_elliptic_solve_host) with the host<->device copies
of the right-hand side, initial guess, residual and solution inside the timed
region.  DOF = E*N^3 per solve (the reference's convention,
examples/kershaw/kershaw.udf).  For the mixed-precision workload the line also
carries the plain FP64 form of the same problem ("fp64_plain": FP64
multigrid and FP64 operator) and the mixed solution's error against it.

    python bench.py [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Under torchrun (N>1) every rank solves its own replica (independent problems,
no data-path collective); `value` sums the ranks' DOFs over the max time.
"""
import argparse
import json
import re
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SCHED7 = "p=7+degree=2,p=3+degree=2,p=1,p=3+degree=2,p=7+degree=2"
PMG = "preconditioner=multigrid;smootherType=cheby+asm;pMGSchedule=" + SCHED7 + ";coarseSolver=jpcg;coarseTol=1e-4"
# mixed-precision headline: optimal 4th-kind Chebyshev over RAS with two algebraic-multigrid V-cycles as
# the coarse solve; degree 6 at the order-7 and order-3 levels with two V-cycles reaches 1e-8 in 22 iterations
# (0.663 s) against 26 / 0.681 s for degree 5 with three V-cycles, 23 / 0.677 s for 6 / 5, 22 / 0.674 s for
# 6 / 7 with one V-cycle, 20 / 0.685 s for 7 / 7 and 31 / 0.705 s for 4 / 5 (GB300, E=48^3); with the Jacobi-PCG
# coarse solve to 1e-4 and degree 5: 26 iterations, 0.714 s
SCHED7_5 = "p=7+degree=5,p=3+degree=5,p=1,p=3+degree=5,p=7+degree=5"
SCHED7_6 = "p=7+degree=6,p=3+degree=6,p=1,p=3+degree=6,p=7+degree=6"
PMG4_JPCG = ("preconditioner=multigrid;smootherType=fourthoptcheby+ras;pMGSchedule=" + SCHED7_5 +
             ";coarseSolver=jpcg;coarseTol=1e-4")
PMG4 = ("preconditioner=multigrid;smootherType=fourthoptcheby+ras;pMGSchedule=" + SCHED7_6 +
        ";coarseSolver=amg;amgIterations=2")
BPS5 = ("solver=pfgmres+nVector=15;residualTol=1e-8+relative;maxIterations=400;preconditioner=multigrid;"
        "smootherType=fourthoptcheby+ras;pMGSchedule=p=7+degree=3,p=3+degree=3,p=1,p=3+degree=3,p=7+degree=3;"
        "mgPrecision=mixed")
FGMRES_NOTE = "the pressure solver's default flexible GMRES(15)"

# name: (elements per side, N, eps, options, description)
WORKLOADS = {
    "kershaw48-n7-mixed": (48, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4 +
                           ";mgPrecision=mixed",
                           "Kershaw box E=48^3 N=7 eps=0.3: FP64 flexible PCG, FP32 pMG 7/3/1 (optimal 4th-kind "
                           "Chebyshev(6)+RAS FDM, coarse solve two algebraic-multigrid V-cycles on the assembled "
                           "order-1 operator), FP64-accurate FP32-pair fine operator, to 1e-8 relative"),
    "kershaw48-n7-mixed-jpcg": (48, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4_JPCG +
                                ";mgPrecision=mixed",
                                "the kershaw48-n7-mixed solve with optimal 4th-kind Chebyshev(5) and the coarse level "
                                "solved by Jacobi-PCG to 1e-4"),
    "kershaw48-n7-mixed-fp16": (48, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4 +
                                ";mgPrecision=mixed;fdmPrecision=fp16",
                                "the kershaw48-n7-mixed solve with the fine-level FDM transforms in FP16 on the tensor "
                                "cores (mma.sync m16n8k16, FP32 accumulation, per-element max-abs scaling)"),
    "kershaw48-n7-mixed-tf32": (48, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4 +
                                ";mgPrecision=mixed;fdmPrecision=tf32",
                                "the kershaw48-n7-mixed solve with the multigrid FDM transforms (orders 7 and 3) in "
                                "TF32 on the tensor cores (order 7 on tcgen05.mma, order 3 on mma.sync m16n8k8)"),
    "kershaw24-n7-mixed-tf32": (24, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4 +
                                ";mgPrecision=mixed;fdmPrecision=tf32",
                                "the kershaw48-n7-mixed-tf32 solve on E=24^3 (profiling size)"),
    "kershaw32-n7-mixed": (32, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4 +
                           ";mgPrecision=mixed", "the kershaw48-n7-mixed solve on E=32^3 (profiling size)"),
    "kershaw16-n7-mixed": (16, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG4 +
                           ";mgPrecision=mixed", "the kershaw48-n7-mixed solve on E=16^3 (profiling size)"),
    "kershaw20-n7-bps5": (20, 7, 0.3, BPS5 + ";coarseSolver=amg;amgIterations=2",
                          "the reference's BPS5 case (examples/kershaw: E=20^3, N=7, eps=0.3, " + FGMRES_NOTE +
                          ", RAS + optimal 4th-kind Chebyshev(3), levels 7/3/1, RHS 3 pi^2 sin(pi x) sin(pi y) "
                          "sin(pi z) on [-0.5,0.5]^3, 1e-8), coarse solve two algebraic-multigrid V-cycles (the "
                          "reference: one BoomerAMG V-cycle); the reference reports 28 iterations"),
    "kershaw20-n7-bps5-jpcg": (20, 7, 0.3, BPS5 + ";coarseSolver=jpcg;coarseTol=1e-4",
                               "the kershaw20-n7-bps5 solve with the coarse level solved by Jacobi-PCG to 1e-4"),
    "kershaw32-n7-fp64": (32, 7, 0.3, "solver=pfcg;residualTol=1e-8+relative;maxIterations=400;" + PMG +
                          ";mgPrecision=fp64;axPrecision=fp64",
                          "Kershaw box E=32^3 N=7 eps=0.3: plain FP64 pMG-PCG (flexible), Chebyshev(2)+ASM, "
                          "coarse Jacobi-PCG 1e-4, to 1e-8 relative"),
    "kershaw16-n7-jacobi": (16, 7, 0.3, "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;"
                            "maxIterations=20000", "Kershaw box E=16^3 N=7 eps=0.3, Jacobi-PCG FP64 to 1e-8"),
    "kershaw8-n7-jacobi": (8, 7, 0.3, "preconditioner=jacobi;solver=pcg;residualTol=1e-8+relative;"
                           "maxIterations=20000", "Kershaw box E=8^3 N=7 eps=0.3, Jacobi-PCG FP64 to 1e-8"),
}
DEFAULT_WORKLOAD = "kershaw48-n7-mixed"
METRIC = "Poisson DOFs/s (E*N^3 / time-to-tolerance)"
# DRAM bytes (read + write) of one launch of the dominant kernel, from an ncu capture of the E=32^3 case of the
# same solve scaled by the element count (every launch streams each element's data once): 273.1 MB at E=32^3
TRAFFIC = {("kershaw48-n7-mixed", "fdm_f32"): 273.1e6 * 3.375}
FP64_PLAIN = {"mgPrecision=mixed": "mgPrecision=fp64;axPrecision=fp64"}


def plain_fp64_options(opts):
    for k, v in FP64_PLAIN.items():
        opts = opts.replace(k, v)
    return opts


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks / throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                power.append(float(r[3]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def dist_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_step_time(t_step):
    """The step time of the whole job: the max of the ranks' step times (each rank solves its own replica;
    the only collective is this scalar reduction, after the timed region)."""
    import torch
    import torch.distributed as dist

    if not dist.is_initialized() or dist.get_world_size() == 1:
        return t_step
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    tt = torch.tensor([t_step], dtype=torch.float64, device=dev)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_value(dofs_per_replica, world, t_step):
    """Whole-job DOF/s: the DOFs of all replicas over the job's step time."""
    return dofs_per_replica * world / t_step


def host_cpu():
    """Host CPU model and the number of threads the oracle uses (all host threads)."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k = line.split(":")[0].strip().lower()
                if k in ("model name", "cpu model"):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
            for line in out.splitlines():
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    threads = int(os.environ.get("OMP_NUM_THREADS", "0")) or os.cpu_count()
    return model or "unknown", threads


def oracle_options(opts):
    """Options for the CPU oracle: its coarse level is always solved by Jacobi-PCG (default 1e-4); the library's
    algebraic-multigrid coarse solve is not restated in the C++ oracle (the reference's own CPU path would run
    BoomerAMG there)."""
    return re.sub(r"coarseSolver=amg(;amgIterations=\d+)?", "coarseSolver=jpcg;coarseTol=1e-4", opts)


def oracle_solves(nel, N, eps, opts, seed, max_solves, budget_s):
    """Complete CPU-oracle solves (all host threads) of the Kershaw-box workload with `nel`^3 elements: setup
    once (not timed), then solves from x = 0 to the workload's tolerance, each with the oracle's own iteration
    count; at least one, then more while the next one fits `budget_s` of solve time and fewer than
    `max_solves` have run.  Returns the solve times and the last solve's info."""
    from oracle import oracle as O
    from nekrs_gb300 import workloads as W

    t0 = time.perf_counter()
    VX, EToV, EToB = W.kershaw_box(nel, eps=eps)
    o = O.Elliptic(N, VX, EToV, EToB, oracle_options(opts))
    rhs = W.box_rhs(N, nel, nel, nel, seed, o.get("ggeo"))
    setup_s = time.perf_counter() - t0
    times, info = [], None
    while True:
        t = time.perf_counter()
        _, info = o.solve(rhs.copy())
        times.append(time.perf_counter() - t)
        if len(times) >= max_solves or sum(times) + times[-1] > budget_s:
            break
    return times, info, setup_s


def cpu_sample(nel, N, eps, opts, budget_s=30.0):
    """The in-line CPU baseline: complete oracle solves of the same solver and options on a Kershaw box of half
    the side (1/8 of the elements), sized to about 10-30 s of CPU work on the host; DOF/s of those complete
    solves, unscaled.  The complete solve at the workload's full size is the reference arm
    (bench.py --impl reference)."""
    nel_s = max(2, nel // 2)
    times, info, setup_s = oracle_solves(nel_s, N, eps, opts, 1234, 3, budget_s)
    model, threads = host_cpu()
    t = float(np.mean(times))
    return {"value": nel_s ** 3 * N ** 3 / t, "unit": "DOF/s", "cores": threads, "kind": "port",
            "cpu_model": model,
            "sample": (f"{len(times)} complete solve(s) of the same solver and options on the {nel_s}^3-element "
                       f"Kershaw box (1/8 of the workload's elements), {info['iterations']} iterations each (the "
                       f"oracle's own count), {t:.1f} s per solve on {threads} host threads; unscaled DOF/s.  "
                       f"The complete {nel}^3 solve is the reference arm's line.  Coarse level: the oracle's "
                       f"Jacobi-PCG to 1e-4"),
            "iterations": int(info["iterations"]), "seconds_per_solve": t, "setup_s": setup_s}


def run_reference(args, nel, N, eps, opts, desc):
    """The reference arm: the CPU oracle (the C++ restatement of the reference's solve, all host threads) on the
    workload itself -- complete solves of the full-size problem to the workload's tolerance, each with the
    oracle's own iteration count.  A complete solve of the E=48^3 headline takes minutes on the host, so this
    arm runs as many complete solves as fit a time budget (at least one) and reports the number it ran as
    `steps`; there is no warm-up on the CPU path."""
    rank, _, _ = dist_info()
    if rank != 0:
        return
    budget = float(os.environ.get("NRSG_REF_BUDGET_S", "240"))
    times, info, setup_s = oracle_solves(nel, N, eps, opts, 1234, max(1, args.steps), budget)
    t = float(np.mean(times))
    value = nel ** 3 * N ** 3 / t
    model, threads = host_cpu()
    line = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": args.gpus, "steps": len(times),
            "warmup": 0, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded Kershaw box, U[-1,1] mass-weighted RHS)", "impl": "reference",
            "config": {"workload": args.workload, "description": desc, "elements": nel ** 3, "N": N,
                       "iterations": int(info["iterations"]), "status": int(info["status"]),
                       "time_to_tolerance_s": t, "setup_s": setup_s, "solve_times_s": times,
                       "requested_steps": args.steps, "requested_warmup": args.warmup,
                       "note": "complete solves of the full-size workload; steps = the solves that fit the time "
                               "budget (NRSG_REF_BUDGET_S, default 240 s); no warm-up on the CPU path"},
            "cpu_baseline": {"value": value, "unit": "DOF/s", "cores": threads, "kind": "port", "cpu_model": model,
                             "sample": f"{len(times)} complete solve(s) of the {nel}^3-element workload to its "
                                       f"tolerance, {info['iterations']} iterations (the oracle's own count; "
                                       f"its coarse level by Jacobi-PCG to 1e-4)"},
            "e2e": {"value": value, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def time_kernel(fn, stream, reps=10):
    import torch

    for _ in range(3):
        fn()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(reps):
        fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / reps


def kernel_rooflines(G, el, N, E):
    """Achieved algorithmic GB/s of the fine-level operator kernels, CUDA events on their stream."""
    import torch

    Np = (N + 1) ** 3
    n = E * Np
    peak, src = load_peaks()
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream
    g64 = torch.from_numpy(el.get("ggeo")).cuda()
    D64 = torch.from_numpy(el.get("D")).cuda()
    q64 = torch.rand(n, dtype=torch.float64, device="cuda")
    a64 = torch.empty_like(q64)
    out = {}
    flops = float(E) * (12 * (N + 1) * Np + 15 * Np + Np)
    t = time_kernel(lambda: G.ax_stored_f64(N, E, g64, D64, 1.0, 0.0, True, q64, a64, cs), stream)
    out["ax_stored_f64"] = {"launch_ms": t * 1e3, "achieved": 64.0 * n / t / 1e9, "unit": "GB/s",
                            "algorithmic_bytes": 64.0 * n, "fp64_tflops": flops / t / 1e12}
    gp = torch.empty(2 * g64.numel(), dtype=torch.float32, device="cuda")
    Dp = torch.empty(2 * D64.numel(), dtype=torch.float32, device="cuda")
    G.split_pairs(g64.numel(), g64, gp, cs)
    G.split_pairs(D64.numel(), D64, Dp, cs)
    t = time_kernel(lambda: G.ax_fp32x2(N, E, gp, Dp, 1.0, 0.0, True, q64, a64, cs), stream)
    out["ax_fp32x2"] = {"launch_ms": t * 1e3, "achieved": 64.0 * n / t / 1e9, "unit": "GB/s",
                        "algorithmic_bytes": 64.0 * n, "fp64_equiv_tflops": flops / t / 1e12}
    del gp
    g32 = g64.float()
    del g64
    D32 = D64.float()
    q32 = q64.float()
    a32 = torch.empty_like(q32)
    t = time_kernel(lambda: G.ax_stored_f32(N, E, g32, D32, 1.0, 0.0, True, q32, a32, cs), stream)
    out["ax_stored_f32"] = {"launch_ms": t * 1e3, "achieved": 32.0 * n / t / 1e9, "unit": "GB/s",
                            "algorithmic_bytes": 32.0 * n}
    if N == 7:
        t = time_kernel(lambda: G.ax_pipe_f32(N, E, g32, D32, 1.0, 0.0, True, q32, a32, cs), stream)
        out["ax_pipe_f32"] = {"launch_ms": t * 1e3, "achieved": 32.0 * n / t / 1e9, "unit": "GB/s",
                              "algorithmic_bytes": 32.0 * n}
        t = time_kernel(lambda: G.ax_const_f32(N, E, g32, D32, 1.0, 0.0, True, q32, a32, cs), stream)
        out["ax_const_f32"] = {"launch_ms": t * 1e3, "achieved": 32.0 * n / t / 1e9, "unit": "GB/s",
                               "algorithmic_bytes": 32.0 * n}
        t = time_kernel(lambda: G.ax_const_prefetch_f32(N, E, g32, D32, 1.0, 0.0, True, q32, a32, cs), stream)
        out["ax_const_prefetch_f32"] = {"launch_ms": t * 1e3, "achieved": 32.0 * n / t / 1e9, "unit": "GB/s",
                                        "algorithmic_bytes": 32.0 * n}
    for v in out.values():
        v["frac_of_hbm"] = v["achieved"] / peak
    return out, peak, src


def fdm_roofline(G, el, N, E, peak, ras, level=0):
    """Achieved algorithmic GB/s of one fused FDM launch of a multigrid level of order N (level 0: the order-7
    Schwarz local solve of the fine level), CUDA events on its stream.  Algorithmic bytes per element follow the
    reference's extended-element formulation (fusedFDM), 4 B each: read u_ext ((N+3)^3), S_x, S_y, S_z
    (3 (N+3)^2) and invL ((N+3)^3), then ASM: write Su_ext ((N+3)^3); RAS: read the weights and write Su on the
    own nodes (2 (N+1)^3)."""
    import torch

    if el.get("mg.bytes")[0] != 4:
        return None
    n = el.mg_level_size(level)
    u = torch.rand(n, dtype=torch.float32, device="cuda")
    su = torch.empty_like(u)
    stream = torch.cuda.current_stream()
    t = time_kernel(lambda: el.mg_fdm(level, u, su), stream)
    nl = N + 3
    per_el = 4.0 * (2 * nl ** 3 + 3 * nl ** 2 + (2 * (N + 1) ** 3 if ras else nl ** 3))
    flops = float(E) * (12 * nl * nl ** 3 + nl ** 3)
    return {"launch_ms": t * 1e3, "achieved": per_el * E / t / 1e9, "unit": "GB/s", "algorithmic_bytes": per_el * E,
            "fp32_tflops": flops / t / 1e12, "frac_of_hbm": per_el * E / t / 1e9 / peak}


COARSE_OPTS = {"jpcg": "coarseSolver=jpcg;coarseTol=1e-4", "amg": "coarseSolver=amg;amgIterations=3"}
BATCH_COARSE = ["jpcg"]  # set from --coarse-solver


def mg_options(N, tol="1e-8"):
    """Mixed-precision pMG-FPCG options for order N (levels N / 3 / 1, or N / 1 for N <= 3), optimal 4th-kind
    Chebyshev(5) + RAS (the degree the E=48^3 solve takes with the Jacobi-PCG coarse solve), coarse solve on the
    assembled order-1 operator (Jacobi-PCG to 1e-4 or three algebraic-multigrid V-cycles, --coarse-solver)."""
    mid = {9: 5, 8: 5, 7: 3, 6: 3, 5: 3, 4: 2}.get(N)
    lv = [N] + ([mid] if mid else []) + [1]
    down = [f"p={q}+degree=5" for q in lv[:-1]]
    sched = ",".join(down + ["p=1"] + down[::-1])
    return (f"solver=pfcg;residualTol={tol}+relative;maxIterations=400;preconditioner=multigrid;"
            f"smootherType=fourthoptcheby+ras;pMGSchedule={sched};{COARSE_OPTS[BATCH_COARSE[0]]};mgPrecision=mixed")


def run_batch(args):
    """Batched solves: independent Poisson problems (cube side U{4..24}, N in {5,7,9}, eps U[0.3,1.0], seeded RHS),
    mixed-precision pMG-FPCG to 1e-8, solved one after another and as one batch stepped one Krylov iteration
    at a time (each problem on its own stream); DOF/s = sum of E*N^3 / wall time."""
    import torch
    import nekrs_gb300 as G
    from nekrs_gb300 import workloads as W

    rng = np.random.default_rng(3)
    K = args.batch_problems
    t0 = time.perf_counter()
    els, rhs, dofs = [], [], 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for k in range(K):
        side, N, eps = int(rng.integers(4, 25)), int(rng.choice([5, 7, 9])), float(rng.uniform(0.3, 1.0))
        VX, EToV, EToB = W.kershaw_box(side, eps=eps)
        el = G.Elliptic(N, VX, EToV, EToB, mg_options(N))
        els.append(el)
        rhs.append(torch.from_numpy(W.box_rhs(N, side, side, side, 1000 + k, el.get("ggeo"))).cuda())
        dofs += side ** 3 * N ** 3
    setup_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    footprint = max(0, free0 - torch.cuda.mem_get_info()[0])
    rs = [torch.empty_like(b) for b in rhs]
    xs = [torch.zeros_like(b) for b in rhs]

    def reset():
        for r, x, b in zip(rs, xs, rhs):
            r.copy_(b)
            x.zero_()
        torch.cuda.synchronize()

    def sequential():
        for el, r, x in zip(els, rs, xs):
            el.solve(r, x)

    out = {}
    for name, fn in (("sequential", sequential), ("batched", lambda: G.solve_batch(els, rs, xs))):
        for _ in range(max(1, args.warmup - 2)):
            reset()
            fn()
        ts = []
        for _ in range(args.steps):
            reset()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        out[name] = float(np.mean(ts))
    its = [el.get("history").size for el in els]
    graphs = [el.get("graph.segments").tolist() for el in els[:2]]
    print(json.dumps({"metric": "batched Poisson DOFs/s (sum of E*N^3 / wall time of the batch)",
                      "value": dofs / out["batched"], "unit": "DOF/s", "n_gpus": 1, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": out["batched"] * 1e3, "higher_is_better": True,
                      "dtype": "f64", "data": "synthetic (seeded Kershaw boxes, U[-1,1] mass-weighted RHS)",
                      "config": {"workload": "batch", "problems": K, "dofs": dofs, "setup_s": setup_s,
                                 "hbm_bytes": int(footprint),
                                 "iterations_min_max": [int(min(its)), int(max(its))],
                                 "graph_segments_first_two": graphs},
                      "sequential": {"value": dofs / out["sequential"], "ms_per_step": out["sequential"] * 1e3},
                      "speedup_batched_vs_sequential": out["sequential"] / out["batched"]}))


def run_velocity(args):
    """Velocity Helmholtz step (the block solve next to the pressure solve): 3 fields on a Kershaw box E=32^3,
    N=7, stress formulation with a variable viscosity field mu(x) and the mass coefficient h = rho bd0 / dt
    (per-node fields, shared by the components), block Jacobi-PCG to 1e-6 relative (nekRS's velocity
    defaults); DOF/s = 3 E N^3 / time-to-tolerance, CUDA events on the solver's stream."""
    import torch
    import nekrs_gb300 as G
    from nekrs_gb300 import workloads as W

    n, N = 32, 7
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    opts = ("solver=pcg+block;preconditioner=jacobi;residualTol=1e-6+relative;maxIterations=1000;poisson=0;"
            "stressFormulation=true")
    t0 = time.perf_counter()
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    x, y, z = (torch.from_numpy(el.get(c)).cuda() for c in ("x", "y", "z"))
    mu = 1.0 + 0.5 * torch.sin(3 * x) * torch.cos(2 * y) + 0.2 * z
    h = torch.full_like(mu, 1.0 * 1.5 / 1e-3)  # rho bd0 / dt with BDF2 bd0 = 3/2, dt = 1e-3
    el.set_coefficients(mu, h, 0)
    setup_s = time.perf_counter() - t0
    g = el.get("ggeo")
    rhs = torch.from_numpy(np.concatenate([W.box_rhs(N, n, n, n, 500 + c, g) for c in range(3)])).cuda()
    r, xs = torch.empty_like(rhs), torch.zeros_like(rhs)

    def step():
        r.copy_(rhs)
        xs.zero_()
        return el.solve(r, xs)

    for _ in range(args.warmup):
        step()
    infos = [step() for _ in range(args.steps)]
    t = float(np.mean([i["solve_ms"] for i in infos])) / 1e3
    dofs = 3 * n ** 3 * N ** 3
    print(json.dumps({"metric": "velocity Helmholtz DOFs/s (3 E N^3 / time-to-tolerance)", "value": dofs / t,
                      "unit": "DOF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": t * 1e3, "higher_is_better": True, "dtype": "f64",
                      "data": "synthetic (seeded Kershaw box, U[-1,1] mass-weighted RHS per component)",
                      "config": {"workload": "velocity", "elements": n ** 3, "N": N, "fields": 3,
                                 "options": opts, "iterations": infos[-1]["iterations"], "setup_s": setup_s,
                                 "status": infos[-1]["status"]}}))


def run_projection(args):
    """Pressure solves of a time-stepping caller: a sequence of right-hand sides that rotate slowly in a
    two-dimensional space (E=32^3, N=7, the mixed-precision pMG-FPCG of the headline, 1e-8 absolute on the
    first solve's residual scale), solved with and without the A-conjugate solution projection
    (residualProjectionVectors 8, start 5): iterations and time per solve over the sequence."""
    import torch
    import nekrs_gb300 as G
    from nekrs_gb300 import workloads as W

    n, N, nsolve = 32, 7, 20
    VX, EToV, EToB = W.kershaw_box(n, eps=0.3)
    base = "solver=pfcg;maxIterations=400;" + PMG4 + ";mgPrecision=mixed"
    probe = G.Elliptic(N, VX, EToV, EToB, base + ";residualTol=1e-8+relative")
    g = probe.get("ggeo")
    b1 = torch.from_numpy(W.box_rhs(N, n, n, n, 71, g)).cuda()
    b2 = torch.from_numpy(W.box_rhs(N, n, n, n, 72, g)).cuda()
    r, x = torch.empty_like(b1), torch.zeros_like(b1)
    r.copy_(b1)
    tol = 1e-8 * probe.solve(r, x)["res0"]
    del probe
    out = {}
    for name, extra in (("none", ""), ("projectionAconj", ";initialGuess=projectionAconj;residualProjectionVectors=8;"
                                                         "residualProjectionStart=5")):
        el = G.Elliptic(N, VX, EToV, EToB, base + f";residualTol={tol}" + extra)
        its, ms = [], []
        for k in range(nsolve):
            r.copy_(float(np.cos(0.1 * k)) * b1 + float(np.sin(0.1 * k)) * b2)
            x.zero_()
            info = el.solve(r, x)
            its.append(info["iterations"])
            ms.append(info["solve_ms"])
        out[name] = {"iterations": its, "ms_per_solve": float(np.mean(ms[5:])), "iterations_after_start":
                     float(np.mean(its[5:]))}
        del el
    dofs = n ** 3 * N ** 3
    t = out["projectionAconj"]["ms_per_solve"] / 1e3
    print(json.dumps({"metric": "Poisson DOFs/s over a solve sequence with solution projection", "value": dofs / t,
                      "unit": "DOF/s", "n_gpus": 1, "steps": nsolve, "warmup": 0, "ms_per_step": t * 1e3,
                      "higher_is_better": True, "dtype": "f64", "data": "synthetic (rotating seeded RHS pair)",
                      "config": {"workload": "projection", "elements": n ** 3, "N": N, "absolute_tol": tol},
                      "sequence": out,
                      "speedup_vs_no_projection": out["none"]["ms_per_solve"] / out["projectionAconj"]["ms_per_solve"]}))


def run_serve(args):
    """Serving loop: Poisson requests with exponential inter-arrival times (mean 2 ms) for `serve_seconds`;
    operators (E log-uniform in [2^9, 2^15], N in {3..9}, eps U[0.3,1.0]) come from a resident pool built
    before the clock starts; each request draws its tolerance from {1e-6, 1e-8, 1e-10} and a seeded RHS.
    Requests are admitted FIFO onto free resident handles while the device footprint of the operators in
    flight stays within an HBM budget, and are stepped together one Krylov iteration at a time; latency =
    completion - arrival.  The same trace is also served one solve at a time."""
    import torch
    import nekrs_gb300 as G
    from nekrs_gb300 import workloads as W

    rng = np.random.default_rng(11)
    P = args.serve_pool
    pool = []
    t0 = time.perf_counter()
    for k in range(P):
        E = float(np.exp(rng.uniform(np.log(2 ** 9), np.log(2 ** 15))))
        side = max(2, int(round(E ** (1.0 / 3.0))))
        N, eps = int(rng.integers(3, 10)), float(rng.uniform(0.3, 1.0))
        VX, EToV, EToB = W.kershaw_box(side, eps=eps)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        el = G.Elliptic(N, VX, EToV, EToB, mg_options(N))
        jw = torch.from_numpy(el.get("ggeo").reshape(side ** 3, 7, -1)[:, 6, :].ravel().copy()).cuda()
        o = {"el": el, "jw": jw, "dofs": side ** 3 * N ** 3, "r": torch.empty_like(jw), "x": torch.empty_like(jw)}
        torch.cuda.synchronize()
        o["bytes"] = max(0, free0 - torch.cuda.mem_get_info()[0])  # device footprint of the operator and its buffers
        pool.append(o)
    setup_s = time.perf_counter() - t0
    # admission by HBM footprint: the operators whose requests are in flight (being stepped, so their working
    # set is hot) may hold at most this many bytes together
    budget = args.serve_hbm_fraction * torch.cuda.mem_get_info()[1]
    # request trace
    mean_gap = args.serve_interarrival_ms / 1e3
    gaps = rng.exponential(mean_gap, size=int(args.serve_seconds / mean_gap * 2) + 16)
    arr = np.cumsum(gaps)
    arr = arr[arr < args.serve_seconds]
    reqs = [{"t": float(t), "op": int(rng.integers(P)), "tol": float(rng.choice([1e-6, 1e-8, 1e-10])),
             "seed": int(rng.integers(1 << 31))} for t in arr]
    gen = torch.Generator(device="cuda")

    def prepare(q):
        o = pool[q["op"]]
        gen.manual_seed(q["seed"])
        o["r"].copy_((torch.rand(o["jw"].numel(), generator=gen, device="cuda", dtype=torch.float64) * 2 - 1)
                     * o["jw"])
        o["x"].zero_()
        o["el"].set_tolerance(q["tol"])

    # warm every handle once
    for o in pool:
        prepare({"op": pool.index(o), "seed": 1, "tol": 1e-8})
        o["el"].solve(o["r"], o["x"])
    torch.cuda.synchronize()

    def serve(concurrent):
        lat = []
        busy = {}  # op -> request handed to the library scheduler
        queue = []
        nxt = 0
        srv = G.Server(budget) if concurrent else None
        start = time.perf_counter()
        while nxt < len(reqs) or queue or busy:
            now = time.perf_counter() - start
            while nxt < len(reqs) and reqs[nxt]["t"] <= now:
                queue.append(reqs[nxt])
                nxt += 1
            if concurrent:
                # requests go to the library (nrsg_server_*) in arrival order once their operator is free
                # (its buffers are reused); the library admits by HBM footprint and steps all in flight
                rest = []
                for q in queue:
                    if q["op"] in busy:
                        rest.append(q)
                        continue
                    prepare(q)
                    o = pool[q["op"]]
                    rid = srv.submit(o["el"], o["r"], o["x"], q["tol"], footprint_bytes=o["bytes"])
                    busy[q["op"]] = (rid, q)
                queue = rest
                srv.step()
                done = {rid for rid, _ in srv.poll()}
                for op in [op for op, (rid, _) in busy.items() if rid in done]:
                    lat.append(time.perf_counter() - start - busy.pop(op)[1]["t"])
            elif queue:
                q = queue.pop(0)
                prepare(q)
                pool[q["op"]]["el"].solve(pool[q["op"]]["r"], pool[q["op"]]["x"])
                lat.append(time.perf_counter() - start - q["t"])
            elif nxt < len(reqs):
                time.sleep(max(0.0, min(1e-3, reqs[nxt]["t"] - now)))
        total = time.perf_counter() - start
        lat = np.array(lat)
        return {"solves": int(lat.size), "solves_per_s": lat.size / total, "wall_s": total,
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3)}

    conc = serve(True)
    seq = serve(False)
    print(json.dumps({"metric": "serving p99 latency (arrival to solution)", "value": conc["p99_ms"], "unit": "ms",
                      "n_gpus": 1, "higher_is_better": False, "dtype": "f64",
                      "data": "synthetic (seeded Kershaw boxes and RHS, exponential arrivals)",
                      "config": {"workload": "serve", "arrivals_s": args.serve_seconds, "requests": len(reqs),
                                 "pool": P, "setup_s": setup_s, "mean_interarrival_ms": args.serve_interarrival_ms,
                                 "pool_bytes": int(sum(o["bytes"] for o in pool)), "inflight_budget_bytes": int(budget)},
                      "concurrent": conc, "sequential": seq,
                      "solves_per_s_vs_sequential": conc["solves_per_s"] / seq["solves_per_s"]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + ["batch", "serve", "velocity", "projection"])
    ap.add_argument("--batch-problems", type=int, default=256, help="problems in the batch workload")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window of the serve workload (config: 60)")
    ap.add_argument("--serve-pool", type=int, default=24, help="resident operators of the serve workload")
    ap.add_argument("--serve-interarrival-ms", type=float, default=2.0,
                    help="mean of the exponential inter-arrival times (config: 2 ms, far above one GPU's capacity "
                         "for this request mix; a larger mean measures latency at a load the GPU sustains)")
    ap.add_argument("--serve-hbm-fraction", type=float, default=0.5,
                    help="HBM share the operators of in-flight requests may hold together (admission)")
    ap.add_argument("--mesh", default=None,
                    help="read the mesh from a Nek5000 .re2 box file (e.g. the reference's kershaw.re2); the "
                         "workload's order, eps and options apply, the right-hand side is the BPS5 one")
    ap.add_argument("--coarse-solver", default="jpcg", choices=["jpcg", "amg"],
                    help="coarse solve of the batch and serve workloads' problems")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--oracle-error", action="store_true",
                    help="also solve the same right-hand side with the CPU oracle in FP64 throughout (FP64 "
                         "multigrid, minutes on the host) and report the GPU solution's error against it")
    ap.add_argument("--no-fp64-plain", action="store_true")
    ap.add_argument("--solve-only", action="store_true",
                    help="time the device-resident solves only (no e2e, FP64 comparison or kernel rooflines)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    BATCH_COARSE[0] = args.coarse_solver
    args.workload_name = args.workload
    if args.workload in ("batch", "serve", "velocity", "projection"):
        import torch

        torch.cuda.set_device(dist_info()[2])
        {"batch": run_batch, "serve": run_serve, "velocity": run_velocity,
         "projection": run_projection}[args.workload](args)
        return
    nel, N, eps, opts, desc = WORKLOADS[args.workload]

    if args.impl == "reference":
        run_reference(args, nel, N, eps, opts, desc)
        return

    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import nekrs_gb300 as G
    from nekrs_gb300 import workloads as W

    if args.mesh:
        from nekrs_gb300 import re2 as R

        VX, EToV, EToB = R.kershaw_mesh_from_re2(args.mesh, eps)
        args.workload_name = f"{args.workload}@{os.path.basename(args.mesh)}"
    else:
        VX, EToV, EToB = W.kershaw_box(nel, eps=eps)
    E = VX.shape[0]
    dofs = E * N ** 3
    t0 = time.perf_counter()
    el = G.Elliptic(N, VX, EToV, EToB, opts)
    setup_s = time.perf_counter() - t0
    if "bps5" in args.workload or args.mesh:
        # kershaw.udf: P0 = 3 pi^2 sin(pi x) sin(pi y) sin(pi z) at every node of the mesh on [-0.5, 0.5]^3
        xs, ys, zs = (el.get(c) - 0.5 for c in ("x", "y", "z"))
        rhs = 3 * np.pi ** 2 * np.sin(np.pi * xs) * np.sin(np.pi * ys) * np.sin(np.pi * zs)
    else:
        rhs = W.box_rhs(N, nel, nel, nel, 1234 + rank, el.get("ggeo"))
    rhs_d = torch.from_numpy(rhs).cuda()
    r = torch.empty_like(rhs_d)
    x = torch.zeros_like(rhs_d)

    def step():
        r.copy_(rhs_d)
        x.zero_()
        return el.solve(r, x)

    for _ in range(args.warmup):
        info = step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = G.kernel_launches()
    infos = []
    torch.cuda.synchronize()
    if args.solve_only:
        torch.cuda.profiler.start()  # a profiler started with capture off records the timed solves only
    for _ in range(args.steps):
        infos.append(step())
    torch.cuda.synchronize()
    if args.solve_only:
        torch.cuda.profiler.stop()
    launches = G.kernel_launches() - l0
    clk = clocks.stop()
    failed = [i["status"] for i in infos if i["status"] != 0]
    if failed:
        raise SystemExit(f"solve failed with status {failed[0]}: {G.last_error() if hasattr(G, 'last_error') else ''}")
    t_step = replica_step_time(float(np.mean([i["solve_ms"] for i in infos])) / 1e3)
    value = job_value(dofs, world, t_step)
    x_mixed = x.cpu().numpy().copy()
    if args.solve_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": t_step * 1e3, "solve_only": True,
                              "config": {"workload": args.workload_name, "iterations": infos[-1]["iterations"],
                                         "coarse_iterations_last_vcycle": el.get("mg.coarseIters").tolist()
                                         if "multigrid" in opts else None},
                              "gpu_launches": int(launches), "clocks": clk}))
        return

    # ---- end to end through the host-buffer C ABI call (pinned host memory)
    rh = torch.from_numpy(rhs.copy()).pin_memory()
    xh = torch.zeros_like(rh).pin_memory()
    e2e_t = []
    for s in range(args.warmup + args.steps):
        rh.copy_(torch.from_numpy(rhs))
        xh.zero_()
        t = time.perf_counter()
        el.solve_host_ptr(rh.data_ptr(), xh.data_ptr())
        if s >= args.warmup:
            e2e_t.append(time.perf_counter() - t)
    e2e_s = float(np.mean(e2e_t))
    del rh, xh

    peak, psrc = load_peaks()
    tuned = None
    if "multigrid" in opts:
        names = ["vec", "plain", "epb2", "pipe", "const", "constpf"]
        ch = el.get("mg.axKernel").astype(int).tolist()
        tm = el.get("mg.axTimes").reshape(len(ch), len(names)) if ch else []
        tuned = [{"level_order": int(o), "chosen": names[c], "ms": {names[k]: (round(float(v), 4) if v > 0 else None)
                                                                    for k, v in enumerate(row)}}
                 for o, c, row in zip(el.get("mg.levels").astype(int).tolist(), ch, tm)]
    fdm = (fdm_roofline(G, el, N, E, peak, "ras" in opts)
           if "multigrid" in opts and ("asm" in opts or "ras" in opts) else None)
    fdm3 = None
    if fdm is not None and "fdmPrecision" not in opts:
        orders = el.get("mg.levels").astype(int).tolist()
        if len(orders) > 2 and orders[1] == 3:
            fdm3 = fdm_roofline(G, el, 3, E, peak, "ras" in opts, level=1)
    extra = {}
    # time-to-tolerance at the other tolerances of the mixed-precision config
    tols = {}
    if "mgPrecision=mixed" in opts and not args.no_fp64_plain:
        for tol in (1e-6, 1e-10):
            el.set_tolerance(tol)
            r.copy_(rhs_d)
            x.zero_()
            it = el.solve(r, x)
            tols[tol] = {"mixed_s": it["solve_ms"] / 1e3, "mixed_iterations": it["iterations"],
                         "x": x.cpu().numpy().copy()}
        el.set_tolerance(1e-8)
    if "mgPrecision=mixed" in opts and not args.no_fp64_plain:
        del el
        torch.cuda.empty_cache()
        elp = G.Elliptic(N, VX, EToV, EToB, plain_fp64_options(opts))
        for _ in range(1):
            r.copy_(rhs_d)
            x.zero_()
            elp.solve(r, x)
        r.copy_(rhs_d)
        x.zero_()
        ip = elp.solve(r, x)
        if ip["status"] != 0:
            raise SystemExit(f"FP64 comparison solve failed with status {ip['status']}")
        xp = x.cpu().numpy()
        extra["fp64_plain"] = {"value": dofs / (ip["solve_ms"] / 1e3), "unit": "DOF/s", "iterations": ip["iterations"],
                               "time_to_tolerance_s": ip["solve_ms"] / 1e3,
                               "options": plain_fp64_options(opts)}
        extra["speedup_mixed_vs_fp64_plain"] = value / world / extra["fp64_plain"]["value"]
        extra["error_vs_fp64"] = float(np.linalg.norm(x_mixed - xp) / np.linalg.norm(xp))
        ttt = {"1e-08": {"mixed_s": t_step, "mixed_iterations": infos[-1]["iterations"],
                         "fp64_s": ip["solve_ms"] / 1e3, "fp64_iterations": ip["iterations"],
                         "error_vs_fp64": extra["error_vs_fp64"]}}
        for tol, v in tols.items():
            elp.set_tolerance(tol)
            r.copy_(rhs_d)
            x.zero_()
            it = elp.solve(r, x)
            xq = x.cpu().numpy()
            ttt[f"{tol:.0e}"] = {"mixed_s": v["mixed_s"], "mixed_iterations": v["mixed_iterations"],
                                 "fp64_s": it["solve_ms"] / 1e3, "fp64_iterations": it["iterations"],
                                 "error_vs_fp64": float(np.linalg.norm(v["x"] - xq) / np.linalg.norm(xq))}
        extra["time_to_tolerance"] = ttt
        del elp
        torch.cuda.empty_cache()
        el = None
    # ---- kernel rooflines (fine-level operator kernels)
    if el is None:
        el = G.Elliptic(N, VX, EToV, EToB, "preconditioner=jacobi")
    kr, peak, psrc = kernel_rooflines(G, el, N, E)
    fdm_name = ("fdm_f16" if "fdmPrecision=fp16" in opts else "fdm_tf32" if "fdmPrecision=tf32" in opts
                else "fdm_f32")
    if fdm is not None:
        kr[fdm_name] = fdm
    if fdm3 is not None:
        kr["fdm_f32_order3"] = fdm3
    # the dominant kernel of the solve by share of device time (ncu launch list of this workload)
    dominant = fdm_name if fdm is not None else ("ax_fp32x2" if "mixed" in opts else "ax_stored_f64")
    d = kr[dominant]
    roof = {"bound": "hbm", "kernel": dominant, "achieved": d["achieved"], "peak": peak, "unit": "GB/s",
            "frac": d["achieved"] / peak, "traffic": TRAFFIC.get((args.workload, dominant)),
            "peak_source": psrc + " (MEASURED_PEAKS.json hbm_gbs)", "launch_ms": d["launch_ms"], "kernels": kr,
            "note": "fdm_f32: the order-7 FP32 Schwarz local solve, algorithmic bytes of the reference's extended-"
                    "element form (fdm_f32_order3: the order-3 level's); FP64 axhelm is FP64-pipe bound on GB300 (1.25 TF/s nominal); ax_fp32x2 is its "
                    "FP64-accurate FP32-pair form (FP32-pipe bound); ax_stored_f32 is the HBM-bound multigrid operator"}

    line = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Kershaw box, U[-1,1] mass-weighted RHS)",
            "config": {"workload": args.workload_name, "description": desc, "elements": E, "N": N,
                       "dofs_per_solve": dofs, "iterations": infos[-1]["iterations"],
                       "time_to_tolerance_s": t_step, "setup_s": setup_s,
                       "l2": "inputs larger than L2 (E-vectors 8*E*Np B, geometric factors 56*E*Np B)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "e2e": {"value": dofs / e2e_s, "unit": "DOF/s", "h2d_bytes_per_step": 2 * rhs.nbytes,
                    "d2h_bytes_per_step": 2 * rhs.nbytes},
            "roofline": roof, "gpu_launches": int(launches), "clocks": clk, "axhelm_autotuner": tuned}
    line.update(extra)
    if rank == 0 and args.oracle_error:
        from oracle import oracle as O

        t0 = time.perf_counter()
        fopts = oracle_options(plain_fp64_options(opts))
        orc = O.Elliptic(N, VX, EToV, EToB, fopts)
        xo, io = orc.solve(rhs.copy())
        line["error_vs_fp64_oracle"] = {
            "value": float(np.linalg.norm(x_mixed - xo) / np.linalg.norm(xo)), "oracle_iterations": int(io["iterations"]),
            "oracle_options": fopts, "oracle_seconds": time.perf_counter() - t0,
            "note": "relative 2-norm difference between the GPU solution of this workload and the CPU oracle's "
                    "FP64-throughout solve (FP64 multigrid) of the same right-hand side at the same tolerance"}
        del orc
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(nel, N, eps, opts)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
