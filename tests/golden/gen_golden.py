"""Generates the golden fixtures of tests/golden/ from the reference's own CPU
evaluator, compiled from the reference sources into oracle/_ref/libmlref.so
(see oracle/Makefile and oracle/ref_driver.cpp).

Run where the reference tree is mounted:
    python tests/golden/gen_golden.py <reference root>

Outputs
  berlin52.json  instances/01_berlin52.tsp as MLProblem loads it (costTour,
                 distRound = false): coordinates, problem size, the
                 MTRandom(0) + random(0.5) start tour, its cost and its full ADS
                 buffer after ldsUpdate(); MTRandom outputs.
  ref_cases.json more instances / seeds / rounding modes: start tour, cost and
                 the sha256 of the ADS buffer (header words 0..5 and the data
                 region; header words 6..31 are uninitialised in the reference).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402


def _p(a):
    return C.c_void_p(a.ctypes.data)


def ads_digest(a: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(a[:6].astype("<u4").tobytes())
    h.update(a[32:].astype("<u4").tobytes())
    return h.hexdigest()


def main(ref_root: str) -> None:
    os.environ["REF_SRC"] = os.path.join(ref_root, "source")
    lib_path = oracle.build_ref()
    if not lib_path:
        raise SystemExit("reference sources not found")
    R = C.CDLL(lib_path)
    R.ref_random_solution.restype = C.c_uint32
    R.ref_lds_update.restype = C.c_uint32
    R.ref_ads_size.restype = C.c_uint32
    inst = lambda name: os.path.join(ref_root, "instances", name).encode()

    def load(name, dist_round):
        n = R.ref_problem_size(inst(name), 1, dist_round)
        x = np.zeros(n, np.int32)
        y = np.zeros(n, np.int32)
        R.ref_problem_weights(inst(name), 1, dist_round, None, _p(x), _p(y))
        return n, x, y

    def solution(name, dist_round, seed):
        n, x, y = load(name, dist_round)
        t = np.zeros(n, np.int32)
        cost = R.ref_random_solution(inst(name), 1, dist_round, seed, C.c_float(0.5), _p(t))
        words = R.ref_ads_size(inst(name), 1, dist_round) // 4
        ads = np.zeros(words, np.uint32)
        c2 = R.ref_lds_update(inst(name), 1, dist_round, _p(t), n, _p(ads))
        assert c2 == cost
        return n, x, y, t, int(cost), ads

    mt = np.zeros(5, np.uint32)
    R.ref_mt_rand(0, 5, _p(mt))
    mt0 = np.zeros(6, np.uint32)
    R.ref_mt_rand(0, 6, _p(mt0))
    mt1 = np.zeros(5, np.uint32)
    R.ref_mt_rand(1, 5, _p(mt1))
    rmax = {}
    for mx in (0, 1, 9, 51, 1000, 4294967294):
        o = np.zeros(16, np.uint32)
        R.ref_mt_rand_max(12345, mx, 16, _p(o))
        rmax[str(mx)] = o.tolist()

    size, x, y, t, cost, ads = solution("01_berlin52.tsp", 0, 0)
    berlin = {
        "source": "instances/01_berlin52.tsp via oracle/_ref (MLProblem::load, MLSolution::random/update/ldsUpdate)",
        "size": size,
        "x": x[: size - 1].tolist(),
        "y": y[: size - 1].tolist(),
        "random_tour_seed0": t.tolist(),
        "cost_random_tour_seed0": cost,
        "ads_random_tour_seed0": ads.tolist(),
        "k4_cost_after_swap_pass": 367403,
        "mt_seed0": mt.tolist(),
        "mt_seed0_mod10": (mt0 % 10).tolist(),
        "mt_seed1_mod10": (mt1 % 10).tolist(),
        "mt_rand_max_seed12345": rmax,
    }
    with open(os.path.join(HERE, "berlin52.json"), "w") as f:
        json.dump(berlin, f)

    cases = []
    for name, dr, seed in [("01_berlin52.tsp", 1, 7), ("02_kroD100.tsp", 0, 500), ("02_kroD100.tsp", 1, 3),
                           ("03_pr226.tsp", 0, 100), ("05_TRP-S500-R1.tsp", 1, 500), ("eil51.tsp", 0, 1),
                           ("st70.tsp", 1, 9)]:
        size, x, y, t, cost, ads = solution(name, dr, seed)
        cases.append({"instance": name, "dist_round": dr, "seed": seed, "size": size,
                      "x": x[: size - 1].tolist(), "y": y[: size - 1].tolist(),
                      "tour": t.tolist(), "cost": cost, "ads_sha256": ads_digest(ads)})
    with open(os.path.join(HERE, "ref_cases.json"), "w") as f:
        json.dump(cases, f)
    print("wrote", os.path.join(HERE, "berlin52.json"), os.path.join(HERE, "ref_cases.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: gen_golden.py <reference root (the directory holding source/ and instances/)>")
    main(sys.argv[1])
