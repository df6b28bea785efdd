"""Benchmark of the GB300 MLP local-search engine (one JSON line on stdout).

Workload (the plain single-instance configuration): n = 1000 nodes with integer
coordinates uniform in [0,1000]^2, TSPLIB EUC_2D nint distances as an int32
n x n matrix resident in HBM, depot 0, seeded random start tours.  One step is
one full multi-improvement DVND (swap, 2-opt, Or-opt-1/2/3) from a new seeded
start tour to its local optimum; every sweep of it evaluates 3,980,527 moves.

Reported:
  value      move evaluations / s over the timed DVND steps (device time, tours
             already resident in HBM, L2 flushed before every step)
  e2e        the same metric through the C-ABI with host buffers (H2D of the
             start tour and D2H of the result inside the timed region)
  roofline   the sweep kernel: algorithmic bytes per sweep / CUDA-event time
  cpu_baseline  the oracle (CPU restatement of the reference path) on the
             host cores, on a bounded sample of the same workload

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "wamca-gpu-mi_gb300"))

METRIC = "move evals/s + DVND solves/s at n=1000 (bit-exact); p50/p99 solve latency"
UNIT = "move evals/s"
N_NODES = 1000
INSTANCE_SEED = 2024
# Algorithmic bytes per move evaluation (distance words + prefix words that vary per move).
BYTES_PER_EVAL = {0: 20, 1: 16, 2: 16, 3: 16, 4: 16}


def blocks(nb: int, size: int) -> int:
    if nb == 0:
        return (size + 1) // 2 - 1
    if nb == 1:
        return (size + 1) // 2
    return size - (nb - 1) - 2


def threads(nb: int, size: int) -> int:
    if nb == 0:
        return size - 4
    if nb == 1:
        return size - 3
    return size - (nb - 1) - 2


def sweep_evals(size: int) -> int:
    return sum(blocks(nb, size) * threads(nb, size) for nb in range(5))


def sweep_bytes(size: int) -> int:
    return sum(blocks(nb, size) * threads(nb, size) * BYTES_PER_EVAL[nb] for nb in range(5))


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic_per_sweep() -> float | None:
    """DRAM bytes per sweep launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "sweep_n1000_ncu.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("dram_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
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
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(vals: list[float], world: int) -> list[float]:
    if world <= 1:
        return vals
    import torch
    import torch.distributed as dist

    t = torch.tensor(vals, dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def reduce_sum(vals: list[float], world: int) -> list[float]:
    if world <= 1:
        return vals
    import torch
    import torch.distributed as dist

    t = torch.tensor(vals, dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.tolist()


# --------------------------------------------------------------------------- CPU
def cpu_baseline(size_n: int, budget_s: float = 12.0) -> dict:
    """The oracle timed on the host cores: full n=1000 sweeps (all threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from mlpgpu import workloads

    x, y = workloads.uniform_instance(size_n, INSTANCE_SEED)
    D = oracle.dist(x, y, True)
    t = workloads.random_perm_tour(size_n, 0)
    cores = os.cpu_count() or 1
    oracle.sweep(t, D, threads=cores)  # warm-up
    t0 = time.perf_counter()
    reps, evals = 0, 0
    while time.perf_counter() - t0 < budget_s and reps < 400:
        evals += oracle.sweep(t, D, threads=cores)[0]
        reps += 1
    dt = time.perf_counter() - t0
    return {"value": evals / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{reps} full neighbourhood sweeps (swap, 2-opt, Or-opt-1/2/3) of the n={size_n} "
                      f"instance, {sweep_evals(size_n + 1)} evals each, oracle with {cores} OpenMP threads"}


def run_reference(args, world, rank) -> None:
    """Reference arm: the reference path's CPU restatement (oracle port) timed on
    the host cores -- full DVND solves of the same workload, all host threads."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from mlpgpu import workloads

    n = N_NODES
    x, y = workloads.uniform_instance(n, INSTANCE_SEED)
    D = oracle.dist(x, y, True)
    cores = os.cpu_count() or 1
    for w in range(args.warmup):
        oracle.dvnd(workloads.random_perm_tour(n, 10_000 + w), D, threads=cores, max_iters=args.ref_iters)
    times, evals, solves = [], 0, 0
    for k in range(args.steps):
        t = workloads.random_perm_tour(n, k)
        t0 = time.perf_counter()
        _, st = oracle.dvnd(t, D, threads=cores, max_iters=args.ref_iters)
        times.append(time.perf_counter() - t0)
        evals += st["evals"]
    total = sum(times)
    value = evals / total
    sample = (f"{args.steps} DVND runs of the n={n} instance from seeded random starts, each capped at "
              f"{args.ref_iters} sweeps, oracle port with {cores} OpenMP threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded uniform coordinates, EUC_2D nint distances)",
        "config": {"workload": "plain DVND n=1000 (swap, 2-opt, Or-opt-1/2/3) from random starts",
                   "n": n, "host_threads": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# --------------------------------------------------------------------------- GPU
def run_ours(args, world, rank, local) -> None:
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    import mlpgpu
    from mlpgpu import workloads

    lib = mlpgpu.lib()
    _ = lib
    mlpgpu._check(mlpgpu.lib().mlp_set_device(local))
    n = N_NODES
    size = n + 1
    x, y = workloads.uniform_instance(n, INSTANCE_SEED)
    prob = mlpgpu.Problem.from_coords(x, y, dist_round=True)
    solver = mlpgpu.Solver(prob, wide=False)
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")  # > 129 MB L2

    # Start tours (a distinct seeded start per step and rank) staged in HBM.
    nsteps = args.warmup + args.steps
    tours = [workloads.random_perm_tour(n, 1_000 * rank + k) for k in range(nsteps)]
    tours_dev = torch.tensor(np.stack(tours), dtype=torch.int32, device="cuda")
    solver.set_tour(tours[0])
    shape = solver.autotune() if args.autotune else None

    # ---- sweep kernel timing (roofline) ----
    ev = sweep_evals(size)
    sb = sweep_bytes(size)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.sweeps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.sweeps)]
    with torch.cuda.stream(stream):
        for _ in range(3):
            solver.sweep(mlpgpu.NB_ALL, 1)
        for r in range(args.sweeps):
            flush.zero_()
            starts[r].record(stream)
            solver.sweep(mlpgpu.NB_ALL, 1)
            ends[r].record(stream)
    torch.cuda.synchronize()
    # mlp_solver_sweep also enqueues a prepare (key reset) after the sweep kernel;
    # time a prepare alone and subtract it to isolate the sweep kernel.
    pst = [torch.cuda.Event(enable_timing=True) for _ in range(args.sweeps)]
    pen = [torch.cuda.Event(enable_timing=True) for _ in range(args.sweeps)]
    with torch.cuda.stream(stream):
        for r in range(args.sweeps):
            flush.zero_()
            pst[r].record(stream)
            solver.sweep(mlpgpu.NB_ALL, 0)
            pen[r].record(stream)
    torch.cuda.synchronize()
    t_sweep_prep = statistics.median(s.elapsed_time(e) for s, e in zip(starts, ends)) * 1e-3
    t_prep = statistics.median(s.elapsed_time(e) for s, e in zip(pst, pen)) * 1e-3
    t_sweep = max(t_sweep_prep - t_prep, 1e-9)

    # ---- DVND steps: device time, tours resident in HBM ----
    step_ms, step_evals, step_sweeps, costs = [], [], [], []
    sampler = ClockSampler(local)
    for k in range(nsteps):
        if k == args.warmup:
            sampler.start()
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            solver.set_tour_device(tours_dev[k].data_ptr())
            solver.dvnd_async(mlpgpu.NB_ALL)
            e1.record(stream)
        torch.cuda.synchronize()
        st = solver.stats()
        if k >= args.warmup:
            step_ms.append(e0.elapsed_time(e1))
            step_evals.append(st["evals"])
            step_sweeps.append(st["sweeps"])
            costs.append(st["cost"])
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = sampler.stop()

    # ---- e2e through the C-ABI with host buffers ----
    host_tours = [torch.from_numpy(t).pin_memory() for t in tours]
    out = torch.empty(size, dtype=torch.int32).pin_memory()
    e2e_s, e2e_evals = [], []
    for k in range(nsteps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mlpgpu._check(mlpgpu.lib().mlp_solver_set_tour(solver._h, mlpgpu.C.c_void_p(host_tours[k].data_ptr()), size))
        st = mlpgpu.DvndStats()
        mlpgpu._check(mlpgpu.lib().mlp_solver_dvnd(solver._h, mlpgpu.NB_ALL, 1 << 20, mlpgpu.C.byref(st)))
        mlpgpu._check(mlpgpu.lib().mlp_solver_get_tour(solver._h, mlpgpu.C.c_void_p(out.data_ptr()), size))
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            e2e_s.append(dt)
            e2e_evals.append(st.evals)
            assert st.cost == costs[k - args.warmup], "e2e and device runs disagree"

    total_s = sum(step_ms) * 1e-3
    agg = reduce_sum([float(sum(step_evals)), float(len(step_ms)), float(sum(e2e_evals))], world)
    tmax = reduce_max([total_s, sum(e2e_s)], world)
    value = agg[0] / tmax[0]
    solves = agg[1] / tmax[0]
    e2e_value = agg[2] / tmax[1]
    if rank != 0:
        return
    lat = sorted(step_ms)
    p = lambda q: lat[min(len(lat) - 1, max(0, math.ceil(q * len(lat)) - 1))]
    peaks = measured_peaks()
    achieved = sb / t_sweep / 1e9
    launches = 0
    for s in step_sweeps:
        body = (s + 1) // 2
        launches += 2 + 5 * body  # prepare + stats, then per loop body: 2 x (sweep + merge) + condition
    traffic = ncu_traffic_per_sweep()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded uniform coordinates in [0,1000]^2, EUC_2D nint int32 distances)",
        "config": {"workload": "plain DVND n=1000 to local optimum (swap, 2-opt, Or-opt-1/2/3), one instance "
                               "per launch, seeded random start per step",
                   "n": n, "evals_per_sweep": ev, "l2": "flushed (256 MB write) before every timed step",
                   "tile_shape": shape, "replicas": world},
        "dvnd_solves_per_s": solves,
        "latency_ms": {"p50": p(0.50), "p99": p(0.99), "mean": statistics.mean(step_ms)},
        "sweeps_per_solve": statistics.mean(step_sweeps),
        "sweep": {"evals": ev, "us": t_sweep * 1e6, "evals_per_s": ev / t_sweep},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": size * 4,
                "d2h_bytes_per_step": size * 4 + 16 * 8},
        "roofline": {"kernel": "k_sweep (all five neighbourhoods)", "bound": "hbm", "achieved": achieved,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "traffic": traffic, "algorithmic_bytes_per_launch": sb,
                     "peak_source": peaks["source"] + " hbm_gbs (STREAM copy)"},
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(n, budget_s=args.cpu_budget)
    print(json.dumps(line))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--sweeps", type=int, default=50)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--ref-iters", type=int, default=1 << 20)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
