#!/usr/bin/env python3
"""Benchmark: time to 1e-4 relative KKT of the GB300 PDHG engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gb300|reference]

One step = one complete solve of the workload LP from its initial point to
relative KKT <= 1e-4 (primal, dual and gap, docs/gpu_pdhg.md:51-57 definitions)
with the mixed-precision restarted adaptive PDHG, the problem already resident
in HBM (handle API).  `value` is the mean device time of a step (CUDA events on
the solver stream, max over ranks); `e2e` is the same solve through the C ABI
entry point with host buffers (conversion, upload, scaling, solve, download and
FP64 KKT packing inside the timed region).

Workloads (seeded synthetic LPs, FP64 data, generators in sih_pdhg.generators):
  zipf-500kx1m   m=500,000 (half equalities), n=1,000,000, 12M nonzeros, column
                 counts Zipf(1.5) clipped to [2, 2000] and rescaled (default)
  random-2kx5k   m=2,000, n=5,000, 8 nonzeros per column
  refinery-168p  one block-angular refinery planning LP of 168 hourly periods
                 (m=149,856, n=237,552, 1.1M nonzeros)
  refinery-512   512 price-shock / outage scenarios of that LP with 24..336
                 periods, solved as one batch (every instance to the tolerance);
                 the line adds the sequential plain-algorithm solves of the same
                 scenarios on the same GPU (sampled) for the batched-vs-plain ratio
  refinery-64    the first 64 of those scenarios (a shorter batch)
  random-2kx5k-x256  256 instances of the 2,000 x 5,000 LP (seeds 0..255) as one batch
  mps:PATH       the LP of an MPS file (sih_pdhg.read_mps); the reference arm prints
                 an `unavailable` line for it (no measured plain iteration count)

Multi-GPU: a single LP is replicated (each rank solves its own copy; scaling
"weak"); a batch workload is partitioned by instance (rank r solves instances
r, r + N, ...; the per-instance results are gathered on the host; scaling
"strong": the whole batch is the job).  No data-path exchange either way.
--impl reference times the reference's algorithm (plain FP32 PDHG) through its
CPU port (oracle/pdhg_oracle.c, OpenMP over all host threads): every timed
step is one complete solve of the workload LP from the initial point until the
FP64 relative KKT of its iterate is <= the tolerance (checked every 100
iterations); warm-up steps run 200 iterations each (page-in, thread start).
Batch workloads time the first scenario's complete solve and scale by nonzeros.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "refinery-optimizer_gb300")
sys.path.insert(0, PKG)

METRIC = "time-to-1e-4 rel. KKT & HBM GB/s: batched mixed vs plain PDHG, 1×GB300"

# Iteration cap of the plain reference algorithm's solves to tolerance (CPU
# arm and the plain comparison on the GPU): on the refinery LPs it does not
# reach 1e-4 within any affordable budget; a capped solve is reported as a
# lower bound.
PLAIN_CAP = {
    "zipf-500kx1m": 200_000,
    "random-2kx5k": 200_000,
    "refinery-168p": 100_000,
    "refinery-512": 100_000,
    "refinery-64": 100_000,
    "random-2kx5k-x256": 200_000,
}

# DRAM bytes per launch of the dominant kernels, read from one ncu capture of
# the same kernels on the same workload (dram__bytes_read.sum + write.sum, mean
# of the first two launches of each in `ncu --metrics dram__bytes_read.sum,
# dram__bytes_write.sum,gpu__time_duration.sum --clock-control none -k
# regex:k_step_ -c 6 python bench.py --profile-solve 64`; summaries in profiles/).
NCU_TRAFFIC_PER_LAUNCH = {
    ("zipf-500kx1m", "k_step_kty"): 117.22e6,
    ("zipf-500kx1m", "k_step_dual"): 112.58e6,
}


# Engine options a workload runs with beyond the defaults (reported in the
# line's `engine_options`): the refinery scenario batches use primal-weight
# smoothing 0.8, which took 358 s for the 512-scenario batch against 441 s with
# PDLP's 0.5 (the slowest scenarios follow the primal weight much better; the
# single 168-period LP is faster with 0.5, 11,904 against 15,232 steps), and one
# lane per column in the A^T y light tasks, the shape the autotuner chose in the
# run where all 512 scenarios reached 1e-4 (the summation order moves the
# trajectories of the slowest scenarios; pinning it makes the run repeatable).
WORKLOAD_OPTIONS = {
    "refinery-512": {"primal_weight_smoothing": 0.8, "lanes_csc": 1},
    "refinery-64": {"primal_weight_smoothing": 0.8, "lanes_csc": 1},
}

WORKLOADS = ["zipf-500kx1m", "random-2kx5k", "refinery-168p", "refinery-512", "refinery-64", "random-2kx5k-x256"]


def make_workload(name: str, seed: int = 0):
    """The workload's LP, or its list of LPs for a batch workload.  ``mps:PATH``
    reads the LP of an MPS file (sih_pdhg.read_mps)."""
    from sih_pdhg.generators import refinery_lp, refinery_scenarios, small_random_lp, zipf_lp

    if name.startswith("mps:"):
        import sih_pdhg

        return sih_pdhg.read_mps(name[4:])
    if name == "zipf-500kx1m":
        return zipf_lp(500_000, 1_000_000, 12_000_000, seed)
    if name == "random-2kx5k":
        return small_random_lp(2000, 5000, 8, seed)
    if name == "refinery-168p":
        return refinery_lp(168, seed)
    if name == "refinery-512":
        return list(refinery_scenarios(512, seed))
    if name == "refinery-64":
        return list(itertools.islice(refinery_scenarios(512, seed), 64))
    if name == "random-2kx5k-x256":
        return [small_random_lp(2000, 5000, 8, 1000 * seed + k) for k in range(256)]
    raise SystemExit(f"unknown workload {name}")


def as_list(w):
    return w if isinstance(w, list) else [w]


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="zipf-500kx1m",
                    help=f"one of {', '.join(WORKLOADS)}, or mps:PATH (the LP of an MPS file)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tol", type=float, default=1e-4)
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--persistent", type=int, default=-1,
                    help="options.persistent of the engine (step form): -1 automatic, 0 graphs, 1 / 2 persistent")
    ap.add_argument("--highs-seconds", type=float, default=60.0,
                    help="single LPs: time limit of the HiGHS IPM baseline on the host cores (0 = skip)")
    ap.add_argument("--plain-sample", type=int, default=8,
                    help="batch workloads: scenarios timed with the plain algorithm for the sequential estimate")
    ap.add_argument("--plain-cap", type=int, default=1_000_000,
                    help="batch workloads: iteration cap of those plain solves")
    ap.add_argument("--profile-solve", type=int, default=0, metavar="STEPS",
                    help="profiling driver: one mixed solve of exactly STEPS steps, kernels launched one by one "
                         "(no CUDA graph), then exit; prints no bench line")
    ap.add_argument("--profile-algorithm", default="mixed", choices=["mixed", "plain"],
                    help="algorithm of --profile-solve: mixed, or plain (the reference's FP32 PDHG)")
    args = ap.parse_args()
    if args.workload not in WORKLOADS and not args.workload.startswith("mps:"):
        ap.error(f"unknown workload {args.workload}")
    return args


def run_profile_solve(args) -> None:
    """A short solve for ncu captures (run it plain first, then under ncu)."""
    import sih_pdhg

    prob = make_workload(args.workload, seed=0)
    cfg = sih_pdhg.GpuPdhgConfig(max_iterations=args.profile_solve, tol_primal=1e-12, tol_dual=1e-12, tol_gap=1e-12)
    algo = sih_pdhg.ALGO_MIXED if args.profile_algorithm == "mixed" else sih_pdhg.ALGO_PLAIN
    sol = sih_pdhg.GpuSolver.solve_ex(prob, cfg, algorithm=algo, use_graph=0, persistent=args.persistent)
    print(f"profile solve: {sol.simplex_iterations} steps, {sol.time_solver_sec * 1e3:.2f} ms device time")


def workload_seed(name: str, rank: int) -> int:
    """Every rank builds the same workload (seed 0): a single LP is solved by
    every rank (replicas), a batch is partitioned by instance (shard)."""
    return 0


def shard(items, rank: int, world: int):
    """Instances of a batch for one rank: rank, rank + world, ... (strided, so
    every rank gets a like mix of scenario sizes); with their batch indices."""
    idx = list(range(rank, len(items), world))
    return [items[i] for i in idx], idx


def gather_instances(rows, world: int):
    """Host gather of the per-instance summaries of every rank's shard (the only
    exchange of the partitioned batch): every rank gets all rows in batch order."""
    if world == 1:
        return sorted(rows, key=lambda r: r["index"])
    import torch.distributed as dist

    parts = [None] * world
    dist.all_gather_object(parts, rows)
    return sorted((r for part in parts for r in part), key=lambda r: r["index"])


def reduce_max(v: float, world: int, device: str) -> float:
    """Max of a per-rank float over the process group (the timing rule)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(vals, world: int, device: str):
    """Element-wise sum of per-rank floats over the process group."""
    if world == 1:
        return list(vals)
    import torch
    import torch.distributed as dist

    t = torch.tensor(list(vals), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(v) for v in t.tolist()]


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


# ------------------------------------------------------------------ clocks
CLOCK_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(prefix="clocks_", suffix=".csv")
        self.proc = None
        self.gpu = gpu_index
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={CLOCK_QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_hbm_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU baselines (oracle = test/baseline only)
def cpu_pdlp_sample(problem, gpu_attempts: int, sample_s: float) -> dict:
    """FP64 CPU port of the same mixed algorithm (oracle/pdlp_oracle.c: its
    SpMVs and elementwise passes on every host thread, as the reference arm
    uses them) on a bounded number of steps, scaled to the GPU's step count."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    oracle.build()
    attempts = 64
    t0 = time.perf_counter()
    oracle.pdlp_solve(problem, max_attempts=attempts, tol=1e-30)
    dt = time.perf_counter() - t0
    while dt < sample_s / 3 and attempts < 4096:
        attempts *= 2
        t0 = time.perf_counter()
        oracle.pdlp_solve(problem, max_attempts=attempts, tol=1e-30)
        dt = time.perf_counter() - t0
    per_step = dt / attempts  # includes scaling and evaluations, amortised
    return {"value": per_step * gpu_attempts, "unit": "s", "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{attempts} steps of the FP64 CPU port of the same algorithm ({dt:.1f} s), "
                      f"scaled to the {gpu_attempts} steps the GPU needed"}


def _highs_child(path: str, conn) -> None:
    """Child process of cpu_highs: solve the LP stored at `path` with scipy HiGHS IPM."""
    import numpy as np
    import scipy.sparse as sp
    from scipy.optimize import linprog

    d = np.load(path)
    A = sp.csc_matrix((d["val"], d["ri"], d["cp"]), shape=(int(d["m"]), int(d["n"])))
    rl, ru = d["rl"], d["ru"]
    eq = rl == ru
    ub = (~eq) & np.isfinite(ru)
    lb = (~eq) & np.isfinite(rl)
    bounds = [(a if np.isfinite(a) else None, b if np.isfinite(b) else None) for a, b in zip(d["cl"], d["cu"])]
    t0 = time.perf_counter()
    r = linprog(d["c"], A_ub=sp.vstack([A[ub], -A[lb]]).tocsc(), b_ub=np.concatenate([ru[ub], -rl[lb]]),
                A_eq=A[eq].tocsc(), b_eq=rl[eq], bounds=bounds, method="highs-ipm")
    conn.send((int(r.status), float(r.fun) if r.status == 0 else None, time.perf_counter() - t0))


def cpu_highs(prob, limit_s: float) -> dict:
    """HiGHS interior point (scipy's linprog, method 'highs-ipm') on the same LP on
    this host's cores: the FP64 solver listed as a CPU baseline for context.  It
    runs in a child process that is stopped after limit_s seconds (HiGHS's own
    time limit is not checked inside a factorisation); a stopped run is
    reported as not finished."""
    import multiprocessing as mp

    import numpy as np

    try:
        import scipy  # noqa: F401
    except ImportError:
        return {"value": None, "unit": "s", "finished": False, "sample": "scipy not installed on this host"}
    p = prob
    sign = 1 if int(p.sense) == 1 else -1
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "lp.npz")
        np.savez(path, m=p.num_rows(), n=p.num_cols(), cp=p.A.csc_col_ptr(), ri=p.A.csc_row_ind(),
                 val=p.A.csc_values(), c=p.c * sign, cl=p.col_lower, cu=p.col_upper, rl=p.row_lower, ru=p.row_upper)
        ctx = mp.get_context("spawn")  # no fork of a process that holds a CUDA context
        recv, send = ctx.Pipe(duplex=False)
        child = ctx.Process(target=_highs_child, args=(path, send))
        child.start()
        res, t_end = None, time.perf_counter() + limit_s
        while time.perf_counter() < t_end:
            if recv.poll(0.25):
                res = recv.recv()
                break
            if not child.is_alive():
                break
        if child.is_alive():
            child.terminate()  # this child only
        child.join(10)
    done = res is not None and res[0] == 0
    return {"value": res[2] if done else None, "unit": "s", "finished": done, "cores": os.cpu_count() or 1,
            "objective": res[1] * sign if done else None,
            "sample": (f"scipy HiGHS IPM on the same LP in a child process, stopped after {limit_s:g} s: "
                       + (f"optimal in {res[2]:.2f} s" if done else "did not finish"))}


def cpu_plain_per_iteration(data, iters: int, threads: int) -> float:
    """Seconds per iteration of the reference algorithm's CPU port
    (oracle_plain_iterations: the four reference kernels, OpenMP) on arrays
    prepared once by oracle.plain_prepare."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    t0 = time.perf_counter()
    oracle.plain_iterations(data, iters, threads)
    return (time.perf_counter() - t0) / iters


# ------------------------------------------------------------------ shared config
def workload_config(name: str, probs, tol: float) -> dict:
    """`config` of both arms' lines (same keys and values, so the two lines
    describe one workload)."""
    nnz = sum(p.num_nonzeros() for p in probs)
    cfg = {"workload": name, "m": sum(p.num_rows() for p in probs), "n": sum(p.num_cols() for p in probs),
           "nnz": nnz, "tol": tol,
           "l2": "working set larger than the 129 MB L2 (no flush needed)" if nnz * 16 > 129e6
           else "working set L2-resident (small LP: latency-bound)"}
    if len(probs) > 1:
        cfg["instances"] = len(probs)
    return cfg


# ------------------------------------------------------------------ reference arm
def run_reference(args) -> None:
    """The reference's algorithm on the host cores: plain FP32 PDHG (its CPU
    port, oracle/pdhg_oracle.c, OpenMP over every host thread).  Each timed
    step is one complete solve from the initial point to FP64 relative KKT <=
    tol (oracle.plain_solve_kkt); a batch workload solves its first scenario
    and scales by the batch's nonzeros.  A solve that hits PLAIN_CAP makes the
    value a lower bound (the line says so)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    work = make_workload(args.workload)
    probs = as_list(work)
    prob = probs[0]
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    oracle.build()
    data = oracle.plain_prepare(prob)
    cap = PLAIN_CAP.get(args.workload, 200_000)
    nnz_scale = sum(p.num_nonzeros() for p in probs) / prob.num_nonzeros()
    for _ in range(args.warmup):  # short: page-in and thread start, not a solve
        oracle.plain_iterations(data, 200, threads)
    times, results = [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = oracle.plain_solve_kkt(data, args.tol, eval_every=100, max_iters=cap, threads=threads)
        times.append((time.perf_counter() - t0) * nnz_scale)
        results.append(r)
    wall = time.perf_counter() - t_wall
    value = statistics.mean(times)
    its = results[-1]["iterations"]
    reached = all(max(r["rel_primal"], r["rel_dual"], r["rel_gap"]) <= args.tol for r in results)
    note = (f"each step one complete solve of the reference algorithm's CPU port ({threads} threads) from its "
            f"initial point to FP64 relative KKT <= {args.tol:g} (checked every 100 iterations): "
            f"{its} iterations" + ("" if reached else f" (cap {cap} hit: a lower bound)"))
    if len(probs) > 1:
        note += f"; scenario 0 solved, x {nnz_scale:.1f} by nonzeros for all {len(probs)} scenarios"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, seed 0)",
            "config": workload_config(args.workload, probs, args.tol),
            "algorithm": "plain FP32 PDHG (reference), CPU port", "iterations": its,
            "rel_kkt": [results[-1]["rel_primal"], results[-1]["rel_dual"], results[-1]["rel_gap"]],
            "reached_tol": reached, "wall_s_per_step": wall / args.steps,
            "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port", "sample": note},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GB300 arm
def run_gb300(args) -> None:
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(local)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(v: float) -> float:
        return reduce_max(v, world, "cuda")

    work = make_workload(args.workload, seed=workload_seed(args.workload, rank))
    batch = isinstance(work, list)
    all_probs = as_list(work)
    # a batch is partitioned by instance over the ranks; a single LP is replicated
    probs, my_index = shard(all_probs, rank, world) if batch else (all_probs, [0])
    tol = args.tol
    cfg = sih_pdhg.GpuPdhgConfig(max_iterations=1_000_000, tol_primal=tol, tol_dual=tol, tol_gap=tol)
    wopts = WORKLOAD_OPTIONS.get(args.workload, {})
    handle = sih_pdhg.PdhgHandle(probs, cfg, algorithm=sih_pdhg.ALGO_MIXED, persistent=args.persistent, **wopts)
    for _ in range(args.warmup):
        handle.run()
    barrier()
    clocks = ClockSampler(local)
    times = []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        times.append(handle.run())
    barrier()
    wall = time.perf_counter() - t_wall
    clock_info = clocks.stop()
    sols = [handle.result(i) for i in range(len(probs))]
    step = max_over_ranks(statistics.mean(times))
    launches = sols[0].kernel_launches * args.steps
    rows = gather_instances([{"index": i, "status": int(s.status), "iterations": int(s.simplex_iterations),
                              "rel": [s.rel_primal, s.rel_dual, s.rel_gap], "objective": s.primal_objective}
                             for i, s in zip(my_index, sols)], world if batch else 1)
    iters = [r["iterations"] for r in rows]

    # roofline of the dominant SpMV kernel (live CUDA-event timing on the solver stream)
    secs, byts = handle.time_kernels(20)
    shape = handle.launch_shape()
    names = (["k_step_primal", "k_step_dual_packed", "k_step_kty_packed"] if shape["packed"]
             else ["k_step_primal", "k_step_dual", "k_step_kty"])
    timed = [k for k in range(3) if secs[k] > 0]  # the packed step has no elementwise kernel
    dom = max(timed, key=lambda k: secs[k])
    peak, peak_src = measured_hbm_peak()
    achieved = byts[dom] / secs[dom] / 1e9
    all_gbs = {names[k]: round(byts[k] / secs[k] / 1e9, 1) for k in timed}
    handle.close()

    # end to end through the C ABI with host buffers (upload .. download inside)
    e2e_times = []
    e2e_sols = None
    for i in range(1 if batch else 2):
        barrier()
        t0 = time.perf_counter()
        e2e_sols = (sih_pdhg.solve_batch(probs, cfg, persistent=args.persistent, **wopts) if batch
                    else [sih_pdhg.solve_gpu_mixed(probs[0], cfg, persistent=args.persistent, **wopts)])
        torch.cuda.synchronize()
        if batch or i > 0 or args.steps <= 1:
            e2e_times.append(time.perf_counter() - t0)
    e2e = max_over_ranks(statistics.mean(e2e_times))
    h2d = sum(int(s.h2d_bytes) for s in e2e_sols)  # per instance: matrix, vectors
    d2h = sum(int(s.d2h_bytes) for s in e2e_sols)
    if batch and world > 1:  # the whole job's bytes: every rank moved its shard
        h2d, d2h = (int(v) for v in reduce_sum([float(h2d), float(d2h)], world, "cuda"))

    if rank != 0:
        return
    cfg_desc = workload_config(args.workload, all_probs, tol)
    line = {
        "metric": METRIC, "value": step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step * 1e3, "higher_is_better": False,
        "scaling": "strong" if batch and world > 1 else "weak",
        "vs_baseline": None, "dtype": "f32+f64",
        "data": (f"MPS file {args.workload[4:]}" if args.workload.startswith("mps:")
                 else "synthetic (seeded generator, seed 0)"),
        "config": cfg_desc,
        "algorithm": "mixed-precision restarted adaptive PDHG",
        "parallelism": (f"instance partition x{world}" if batch and world > 1 else f"replicas x{world}"),
        "iterations": max(iters), "restarts": sols[0].restarts,
        "status": max(r["status"] for r in rows),
        "rel_kkt": [max(r["rel"][k] for r in rows) for k in range(3)],
        "wall_s_per_step": wall / args.steps,
        "clocks": clock_info,
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "launch_shape": shape,
        "engine_options": wopts,
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_src,
                     "traffic": NCU_TRAFFIC_PER_LAUNCH.get((args.workload, names[dom])),
                     "algorithmic_bytes_per_launch": byts[dom], "all_kernels_gbs": all_gbs},
    }
    if not batch:
        line["plain_gpu"] = plain_gpu_time(probs[0], tol, PLAIN_CAP.get(args.workload, 200_000))
    if not batch:
        line["cusparse_yardstick"] = cusparse_yardstick(probs[0])
    if batch:
        line["iterations_per_instance"] = {"min": min(iters), "median": int(statistics.median(iters)),
                                           "max": max(iters)}
        line["plain_gpu_sequential"] = plain_sequential_sample(all_probs, tol, args.plain_sample, args.plain_cap)
    # CPU baseline: the FP64 port of the same algorithm on one instance, scaled
    # to the whole job by nonzero-steps
    big = 0
    cb = cpu_pdlp_sample(all_probs[big], iters[big], args.cpu_sample_seconds)
    if batch:
        work_all = sum(it * p.num_nonzeros() for it, p in zip(iters, all_probs))
        scale = work_all / (iters[big] * all_probs[big].num_nonzeros())
        cb["value"] *= scale
        cb["sample"] += (f"; x {scale:.1f} to cover all {len(all_probs)} instances "
                         f"(sum over instances of steps x nonzeros)")
    line["cpu_baseline"] = cb
    if not batch and args.highs_seconds > 0:
        line["cpu_highs"] = cpu_highs(all_probs[0], args.highs_seconds)
    print(json.dumps(line), flush=True)


def cusparse_yardstick(prob, reps: int = 20) -> dict:
    """cuSPARSE SpMV (through torch's CSR matrix-vector product) on the same
    matrix, FP32: A x and A^T y as plain SpMVs, GB/s by the same algorithmic
    bytes as the engine's (8 nnz + 4 (segments + 1) + 4 gathered + 4 written per
    segment).  A yardstick only; the engine does not use it."""
    import numpy as np
    import torch

    A = prob.A
    m, n, nnz = prob.num_rows(), prob.num_cols(), prob.num_nonzeros()
    dev = torch.device("cuda")
    i32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(dev)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)
    csr = torch.sparse_csr_tensor(i32(A.csr_row_ptr()), i32(A.csr_col_ind()), f32(A.csr_values()), size=(m, n))
    csc_as_csr = torch.sparse_csr_tensor(i32(A.csc_col_ptr()), i32(A.csc_row_ind()), f32(A.csc_values()), size=(n, m))
    x = torch.rand(n, 1, device=dev)
    y = torch.rand(m, 1, device=dev)
    out = {}
    for name, mat, vec, segs, gathered in (("A_x", csr, x, m, n), ("AT_y", csc_as_csr, y, n, m)):
        for _ in range(3):
            torch.mm(mat, vec)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            torch.mm(mat, vec)
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3 / reps
        byts = 8.0 * nnz + 4.0 * (segs + 1) + 4.0 * gathered + 4.0 * segs
        out[name] = {"us": round(sec * 1e6, 1), "gbs": round(byts / sec / 1e9, 1)}
    out["note"] = "torch CSR matrix-vector product (cuSPARSE), int32 indices, FP32 values; not part of the engine"
    return out


def plain_gpu_time(prob, tol: float, cap: int) -> dict:
    """The reference algorithm (plain FP32 PDHG) on this GPU, solved to relative
    KKT <= tol: runs from the initial point with its own stopping test off
    (zero tolerances) for 1,000, 2,000, 4,000, ... iterations until one reaches
    tol, then bisection between the last two to 5 %; `value` is the device
    time of the shortest run that reached tol (a lower bound when none did
    within `cap`)."""
    import sih_pdhg

    def run(its):
        cfg = sih_pdhg.GpuPdhgConfig(max_iterations=its, tol_primal=0.0, tol_dual=0.0, tol_gap=0.0)
        sol = sih_pdhg.solve_gpu_pdhg(prob, cfg)
        return max(sol.rel_primal, sol.rel_dual, sol.rel_gap) <= tol, sol.time_solver_sec

    run(1000)  # warm-up
    lo, hi, hi_t, its = 0, None, None, 1000
    while True:
        ok, t = run(its)
        if ok:
            hi, hi_t = its, t
            break
        lo = its
        if its >= cap:
            return {"value": t, "unit": "s", "lower_bound": True, "iterations_to_tol": None,
                    "sample": f"the plain path (sih_pdhg_solve) did not reach {tol:g} within {cap} iterations "
                              f"({t:.2f} s device time)"}
        its = min(cap, its * 2)
    while hi - lo > max(100, hi // 20):
        mid = (lo + hi) // 2
        ok, t = run(mid)
        if ok:
            hi, hi_t = mid, t
        else:
            lo = mid
    return {"value": hi_t, "unit": "s", "lower_bound": False, "iterations_to_tol": hi,
            "per_iteration_s": hi_t / hi,
            "sample": f"device time of the plain path (sih_pdhg_solve) run for {hi} iterations, the fewest "
                      f"(to 5 %) whose returned point reaches relative KKT <= {tol:g}"}


def plain_sequential_sample(probs, tol: float, count: int, cap: int = 1_000_000) -> dict:
    """The reference algorithm (plain FP32 PDHG) on the same GPU, one scenario
    after another: for `count` scenarios (evenly spaced through the batch) the
    iterations it needs to reach relative KKT <= tol (its own, weaker stopping
    test off: runs of 2,000, 4,000, ... iterations up to `cap`, the first that
    reaches the tolerance counts) and the device time of that run; the estimate
    for all scenarios scales the sampled seconds by the batch's nonzeros.  A
    scenario that does not reach the tolerance within `cap` contributes the
    time of the capped run, and the estimate is then a lower bound."""
    import sih_pdhg

    pick = sorted(set(int(round(k)) for k in [i * (len(probs) - 1) / max(1, count - 1) for i in range(count)]))
    secs, nnz_s, reached, its_list = 0.0, 0, 0, []
    for i in pick:
        p = probs[i]
        its = 2000
        while True:
            cfg = sih_pdhg.GpuPdhgConfig(max_iterations=its, tol_primal=0.0, tol_dual=0.0, tol_gap=0.0)
            sol = sih_pdhg.solve_gpu_pdhg(p, cfg)
            ok = max(sol.rel_primal, sol.rel_dual, sol.rel_gap) <= tol
            if ok or its >= cap:
                break
            its = min(cap, its * 2)
        secs += sol.time_solver_sec
        nnz_s += p.num_nonzeros()
        reached += int(ok)
        its_list.append(its if ok else None)
    total_nnz = sum(p.num_nonzeros() for p in probs)
    est = secs * total_nnz / max(1, nnz_s)
    return {"value": est, "unit": "s", "lower_bound": reached < len(pick), "iterations_to_tol": its_list,
            "sample": f"{len(pick)} scenarios solved one after another with the plain algorithm, its own stopping "
                      f"test off, until relative KKT <= {tol:g} (runs of 2,000, 4,000, ... iterations, cap {cap}); "
                      f"{reached} reached it; {secs:.2f} s device time scaled by nonzeros to all {len(probs)} "
                      f"scenarios"}


def main() -> None:
    args = parse_args()
    if args.profile_solve > 0:
        run_profile_solve(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
