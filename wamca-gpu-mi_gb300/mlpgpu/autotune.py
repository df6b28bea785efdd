"""Autotuner of the sweep tile shape per tour-size bucket.

The fused sweep evaluates all five neighbourhoods in one kernel, so the tuned
knob is its tile shape (diagonals x rows, 10 compiled shapes), chosen per
bucket of tour sizes and separately for one job (latency: a plain DVND) and
for many jobs sharing the launches (throughput: batches and the server).
Each candidate is timed on real DVND iterations (improving-only sweeps, the
merge, warm L2) from the same seeded start, best of a few repeats; the merge
is the same for every shape, so the differences are the sweep's.

    python -m mlpgpu.autotune [--out FILE] [--sizes 100,200,...]

writes {"device": ..., "table": [[max_size, shape_one, shape_many], ...]}
(max_size = n + 1, the tour length), which mlpgpu loads at start-up
(mlp_tuning_load from C).  Results never depend on the table.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import mlpgpu  # noqa: E402
    from mlpgpu import workloads  # noqa: E402
else:
    from . import workloads
    import mlpgpu

DEFAULT_SIZES = (100, 200, 400, 700, 1000, 1500, 2000, 4000, 10000)


def _best(times: dict) -> int:
    return min(times, key=times.get)


def time_one(n: int, shapes=range(mlpgpu.NUM_TILE_SHAPES), iters: int = 24, reps: int = 3) -> dict:
    """Seconds of `iters` DVND iterations of one job of n nodes, per shape."""
    x, y = workloads.uniform_instance(n, 7)
    p = mlpgpu.Problem.from_coords(x, y)
    s = mlpgpu.Solver(p, wide=n > 5000)
    t = workloads.random_perm_tour(n, 7)
    out = {}
    for sh in shapes:
        s.set_tile_shape(sh)
        best = float("inf")
        for r in range(reps + 1):
            s.set_tour(t)
            t0 = time.perf_counter()
            s.dvnd(max_iters=iters)
            dt = time.perf_counter() - t0
            if r > 0:
                best = min(best, dt)
        out[sh] = best
    return out


def time_many(n: int, shapes=range(mlpgpu.NUM_TILE_SHAPES), iters: int = 12, reps: int = 2) -> dict:
    """Seconds of `iters` DVND iterations of a batch of many jobs of n nodes, per shape."""
    jobs = int(min(256, max(8, 3e8 // (n * n))))
    x, y = workloads.clustered_instance(n, 11)
    p = mlpgpu.Problem.from_coords(x, y)
    b = mlpgpu.Batch(wide=n > 5000)
    for q in range(jobs):
        b.add(p, workloads.random_perm_tour(n, 100 + q))
    out = {}
    for sh in shapes:
        b.set_tile_shape(sh)
        best = float("inf")
        for r in range(reps + 1):
            b.reset()
            t0 = time.perf_counter()
            b.run(max_iters=iters)
            dt = time.perf_counter() - t0
            if r > 0:
                best = min(best, dt)
        out[sh] = best
    b.close()
    return out


def tune(sizes=DEFAULT_SIZES, verbose: bool = True) -> dict:
    rows, detail = [], []
    for n in sizes:
        one = time_one(n, iters=24 if n <= 4000 else 6)
        many = time_many(n, iters=12 if n <= 4000 else 3)
        rows.append([int(n) + 1, _best(one), _best(many)])
        detail.append({"n": int(n), "one_s": {str(k): v for k, v in one.items()},
                       "many_s": {str(k): v for k, v in many.items()}})
        if verbose:
            print(f"n={n}: one job -> shape {rows[-1][1]}, many jobs -> shape {rows[-1][2]}", flush=True)
    dev = "unknown"
    try:
        import torch

        dev = torch.cuda.get_device_name(0)
    except Exception:
        pass
    return {"device": dev, "shapes": "0..13 = 32x4, 32x8, 32x16, 64x4, 64x8, 64x16, 128x8, 128x16, 32x32, 64x32 "
                                      "(diagonals x rows), then 64x8, 64x16, 64x32, 128x16 with two diagonals per "
                                      "thread in the DVND sweep",
            "table": rows, "timings": detail}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--sizes", default=",".join(str(v) for v in DEFAULT_SIZES))
    args = ap.parse_args()
    mlpgpu.set_tuning_table([])  # time every shape explicitly, whatever table was loaded
    res = tune([int(v) for v in args.sizes.split(",")])
    text = json.dumps(res, indent=1)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text + "\n")
    else:
        print(text)


if __name__ == "__main__":
    main()
