"""ctypes wrapper of the oracle (oracle/liboracle.so) -- TEST INFRASTRUCTURE.

The oracle is the CPU restatement of the reference's MLP local-search path
(see mlp_oracle.h).  Only tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py use it, always as the checker or the timed CPU baseline; the
GPU engine never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libmlref.so")

_lib: Optional[C.CDLL] = None


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, f) for f in ("mlp_oracle.cpp", "mlp_oracle.h", "Makefile")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB


REF_DIR = os.path.join(HERE, "_ref")
REF_CUBINS = [os.path.join(REF_DIR, f"ref_{u}.cubin") for u in ("mlkswap", "mlk2opt", "mlkoropt")]
REF_LAUNCH = os.path.join(REF_DIR, "libref_launch.so")


def build_ref(ref_src: Optional[str] = None) -> Optional[str]:
    """Compiles the reference's CPU evaluator and its GPU neighbourhood kernels
    (sm_103a cubins) into _ref/ from the reference's source/ directory
    `ref_src` (else the REF_SRC environment variable; skipped when neither is
    given), and the launcher of those kernels wherever the cubins are (they
    travel with the tree); returns the CPU evaluator's path or None."""
    ref_src = ref_src or os.environ.get("REF_SRC")
    if ref_src and not os.path.isdir(ref_src):
        raise FileNotFoundError(f"reference sources not found: {ref_src}")
    if ref_src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={ref_src}"], check=True)
        subprocess.run(["make", "-s", "-C", HERE, "refgpu", f"REF_SRC={ref_src}"], check=True)
    if all(os.path.exists(c) for c in REF_CUBINS):
        subprocess.run(["make", "-s", "-C", HERE, "reflaunch"], check=True)
    return REF_LIB if os.path.exists(REF_LIB) else None


_ref_gpu: Optional[C.CDLL] = None


def ref_gpu() -> Optional[C.CDLL]:
    """The launcher of the reference's own GPU kernels (oracle/ref_launch.cpp),
    initialised on the current device; None where they were not built."""
    global _ref_gpu
    if _ref_gpu is None:
        if not (os.path.exists(REF_LAUNCH) and all(os.path.exists(c) for c in REF_CUBINS)):
            return None
        L = C.CDLL(REF_LAUNCH)
        L.rl_error.restype = C.c_char_p
        L.rl_init.argtypes = [C.c_char_p]
        L.rl_eval.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_uint64, C.c_int, C.POINTER(C.c_float),
                              C.POINTER(C.c_int), C.POINTER(C.c_int)]
        if L.rl_init(REF_DIR.encode()) != 0:
            raise RuntimeError("reference kernels: " + L.rl_error().decode())
        _ref_gpu = L
    return _ref_gpu


def ref_gpu_eval(nb: int, ads_dev: int, size: int, moves_dev: int, reps: int = 1):
    """Runs the reference's ODC kernel of nb (0 swap, 1 2-opt, 2..4 Or-opt-1..3)
    over the device MLADSData buffer; returns (ms per launch, block, grid)."""
    L = ref_gpu()
    ms, blk, grd = C.c_float(), C.c_int(), C.c_int()
    if L.rl_eval(nb, ads_dev, size, moves_dev, reps, C.byref(ms), C.byref(blk), C.byref(grd)) != 0:
        raise RuntimeError("reference kernel: " + L.rl_error().decode())
    return ms.value, blk.value, grd.value


def decode_move_pack(w: np.ndarray):
    """MLMovePack words (source/mlads.h:180-215): (cost, id, i, j)."""
    w = np.asarray(w, dtype=np.uint64)
    cost = (w >> np.uint64(32)).astype(np.uint32).view(np.int32).astype(np.int64)
    low = (w & np.uint64(0xffffffff)).astype(np.uint32)
    return cost, (low & 0xF).astype(np.int32), ((low >> 4) & 0x3FFF).astype(np.int32), (low >> 18).astype(np.int32)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        sig = {
            "orc_mt_rand": (None, [C.c_uint32, i32, vp]),
            "orc_mt_rand_max": (None, [C.c_uint32, C.c_uint32, i32, vp]),
            "orc_tsplib_read": (i32, [C.c_char_p, i32, vp, vp]),
            "orc_dist_from_coords": (None, [i32, vp, vp, i32, vp]),
            "orc_random_tour": (None, [i32, vp, i32, C.c_uint32, C.c_float, vp]),
            "orc_random_tour_canonical": (None, [i32, vp, C.c_uint32, C.c_float, vp]),
            "orc_cost": (i64, [i32, vp, i32, vp, i32, vp]),
            "orc_ads_build": (None, [i32, vp, i32, vp, vp, vp, i32, i32, vp]),
            "orc_num_blocks": (i32, [i32, i32]),
            "orc_num_threads": (i32, [i32, i32]),
            "orc_eval": (None, [i32, i32, vp, i32, vp, i32, i32, vp, vp, vp, vp]),
            "orc_move_delta_bruteforce": (i64, [i32, i32, i32, i32, vp, i32, vp, i32]),
            "orc_move_delta": (i64, [i32, i32, i32, i32, vp, i32, vp, i32]),
            "orc_can_merge_same": (i32, [i32, i32, i32, i32, i32, i32, i32]),
            "orc_can_merge": (i32, [i32, i32, i32, i32, i32, i32]),
            "orc_merge_same": (i32, [i32, i32, vp, vp, vp, vp]),
            "orc_merge_cross": (i32, [i32, vp, vp, vp, vp, vp]),
            "orc_apply": (None, [i32, i32, i32, i32, vp]),
            "orc_pass": (i32, [i32, i32, vp, i32, vp, i32, i32, vp, vp, vp, vp, vp]),
            "orc_dvnd": (i32, [i32, vp, i32, vp, i32, i32, vp, i32, i32, vp, vp, vp]),
            "orc_sweep": (i64, [i32, vp, i32, vp, i32, i32, vp, i32, vp, vp, vp]),
            "orc_total_select": (i32, [i32, i32, vp, i32, vp, i32, i32, vp, vp, vp, vp]),
            "orc_total_pass": (i32, [i32, i32, vp, i32, vp, i32, i32, vp, vp, vp, vp, vp]),
            "orc_dvnd_total": (i32, [i32, vp, i32, vp, i32, i32, vp, i32, vp, vp, vp]),
            "orc_legacy_no_conflict": (i32, [i32, i32, i32, i32, i32, i32]),
            "orc_legacy_better_no_conflict": (i32, [i32, vp, vp, vp, vp, vp, vp, i32, i32]),
            "orc_legacy_apply_moves": (C.c_uint32, [i32, vp, i32, vp, i32, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def mt_rand(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, np.uint32)
    lib().orc_mt_rand(seed, count, _p(out))
    return out


def mt_rand_max(seed: int, mx: int, count: int) -> np.ndarray:
    out = np.zeros(count, np.uint32)
    lib().orc_mt_rand_max(seed, mx, count, _p(out))
    return out


def read_tsplib(path: str, maxn: int = 20000):
    x = np.zeros(maxn, np.int32)
    y = np.zeros(maxn, np.int32)
    n = lib().orc_tsplib_read(path.encode(), maxn, _p(x), _p(y))
    if n < 0:
        raise IOError(f"tsplib read failed ({n}): {path}")
    return x[:n].copy(), y[:n].copy()


def dist(x, y, dist_round: bool) -> np.ndarray:
    x, y = _i32(x), _i32(y)
    n = len(x)
    D = np.zeros((n, n), np.int32)
    lib().orc_dist_from_coords(n, _p(x), _p(y), int(dist_round), _p(D))
    return D


def random_tour(D: np.ndarray, seed: int, alpha: float = 0.5) -> np.ndarray:
    D = _i32(D)
    n = D.shape[0]
    t = np.zeros(n + 1, np.int32)
    lib().orc_random_tour(n, _p(D), 1, seed, C.c_float(alpha), _p(t))
    return t


def random_tour_canonical(D: np.ndarray, seed: int, alpha: float = 0.5) -> np.ndarray:
    """MLSolution::random with equal distances ordered by client id."""
    D = _i32(D)
    n = D.shape[0]
    t = np.zeros(n + 1, np.int32)
    lib().orc_random_tour_canonical(n, _p(D), seed, C.c_float(alpha), _p(t))
    return t


def cost(tour, D, wide: bool = False) -> int:
    t, D = _i32(tour), _i32(D)
    return int(lib().orc_cost(len(t), _p(t), D.shape[0], _p(D), int(wide), None))


def weights(tour, D) -> np.ndarray:
    t, D = _i32(tour), _i32(D)
    w = np.zeros(len(t), np.int32)
    lib().orc_cost(len(t), _p(t), D.shape[0], _p(D), 0, _p(w))
    return w


def ads(tour, D, x, y, dist_round: bool) -> np.ndarray:
    t, D, x, y = _i32(tour), _i32(D), _i32(x), _i32(y)
    size = len(t)
    out = np.zeros(32 + size * (size + 3), np.uint32)
    lib().orc_ads_build(size, _p(t), D.shape[0], _p(D), _p(x), _p(y), 1, int(dist_round), _p(out))
    return out


def num_blocks(nb: int, size: int) -> int:
    return int(lib().orc_num_blocks(nb, size))


def num_threads(nb: int, size: int) -> int:
    return int(lib().orc_num_threads(nb, size))


def evals_per_sweep(size: int, nbs: Sequence[int] = range(5)) -> int:
    return sum(num_blocks(nb, size) * num_threads(nb, size) for nb in nbs)


def eval_nb(nb: int, tour, D, wide: bool = False, faithful: bool = False):
    t, D = _i32(tour), _i32(D)
    m = num_blocks(nb, len(t))
    c = np.zeros(m, np.int64)
    i = np.zeros(m, np.int32)
    j = np.zeros(m, np.int32)
    ctx = np.zeros(m, np.int32)
    lib().orc_eval(nb, len(t), _p(t), D.shape[0], _p(D), int(wide), int(faithful), _p(c), _p(i), _p(j), _p(ctx))
    return c, i, j, ctx


def move_delta(mid: int, i: int, j: int, tour, D, wide: bool = False, brute: bool = False) -> int:
    t, D = _i32(tour), _i32(D)
    f = lib().orc_move_delta_bruteforce if brute else lib().orc_move_delta
    return int(f(mid, i, j, len(t), _p(t), D.shape[0], _p(D), int(wide)))


def can_merge(m1, m2) -> bool:
    return bool(lib().orc_can_merge(m1[0], m1[1], m1[2], m2[0], m2[1], m2[2]))


def can_merge_same(nb: int, m1, m2) -> bool:
    return bool(lib().orc_can_merge_same(nb, m1[0], m1[1], m1[2], m2[0], m2[1], m2[2]))


def merge_same(nb: int, cost, mi, mj) -> np.ndarray:
    c = np.ascontiguousarray(cost, np.int64)
    mi, mj = _i32(mi), _i32(mj)
    kept = np.zeros(len(c), np.int32)
    k = lib().orc_merge_same(nb, len(c), _p(c), _p(mi), _p(mj), _p(kept))
    return kept[:k].copy()


def merge_cross(ids, mi, mj, cost) -> np.ndarray:
    ids, mi, mj = _i32(ids), _i32(mi), _i32(mj)
    c = np.ascontiguousarray(cost, np.int64)
    kept = np.zeros(len(c), np.int32)
    k = lib().orc_merge_cross(len(c), _p(ids), _p(mi), _p(mj), _p(c), _p(kept))
    return kept[:k].copy()


def apply(mid: int, i: int, j: int, tour: np.ndarray) -> None:
    assert tour.dtype == np.int32 and tour.flags.c_contiguous
    lib().orc_apply(mid, i, j, len(tour), _p(tour))


def pass_(nb: int, tour, D, wide: bool = False, max_moves: int = 1 << 15):
    t, D = _i32(tour).copy(), _i32(D)
    ids = np.zeros(max_moves, np.int32)
    i = np.zeros(max_moves, np.int32)
    j = np.zeros(max_moves, np.int32)
    c = np.zeros(max_moves, np.int64)
    nc = C.c_int64()
    k = lib().orc_pass(nb, len(t), _p(t), D.shape[0], _p(D), int(wide), max_moves, _p(ids), _p(i), _p(j), _p(c),
                       C.byref(nc))
    kk = min(k, max_moves)
    return t, nc.value, list(zip(ids[:kk].tolist(), i[:kk].tolist(), j[:kk].tolist(), c[:kk].tolist()))


def dvnd(tour, D, wide: bool = False, nbs: Sequence[int] = range(5), max_iters: int = 1 << 20,
         threads: int = 1):
    t, D = _i32(tour).copy(), _i32(D)
    nbs_a = _i32(list(nbs))
    fc, ev, mv = C.c_int64(), C.c_int64(), C.c_int64()
    it = lib().orc_dvnd(len(t), _p(t), D.shape[0], _p(D), int(wide), len(nbs_a), _p(nbs_a), max_iters, threads,
                        C.byref(fc), C.byref(ev), C.byref(mv))
    return t, {"cost": fc.value, "iterations": it, "evals": ev.value, "moves": mv.value}


def total_select(nb: int, tour, D, wide: bool = False):
    """Kept moves [(cost, i, j)] of the TOTAL greedy of nb, in greedy order,
    and the number of improving candidates."""
    t, D = _i32(tour), _i32(D)
    cap = 2 * len(t) + 8
    c = np.zeros(cap, np.int64)
    i = np.zeros(cap, np.int32)
    j = np.zeros(cap, np.int32)
    nc = C.c_int64()
    k = lib().orc_total_select(nb, len(t), _p(t), D.shape[0], _p(D), int(wide), cap, _p(c), _p(i), _p(j),
                               C.byref(nc))
    return list(zip(c[:k].tolist(), i[:k].tolist(), j[:k].tolist())), nc.value


def total_pass(nb: int, tour, D, wide: bool = False, max_moves: int = 1 << 15):
    t, D = _i32(tour).copy(), _i32(D)
    ids = np.zeros(max_moves, np.int32)
    i = np.zeros(max_moves, np.int32)
    j = np.zeros(max_moves, np.int32)
    c = np.zeros(max_moves, np.int64)
    nc = C.c_int64()
    k = lib().orc_total_pass(nb, len(t), _p(t), D.shape[0], _p(D), int(wide), max_moves, _p(ids), _p(i), _p(j),
                             _p(c), C.byref(nc))
    kk = min(k, max_moves)
    return t, nc.value, list(zip(ids[:kk].tolist(), i[:kk].tolist(), j[:kk].tolist(), c[:kk].tolist()))


def dvnd_total(tour, D, wide: bool = False, nbs: Sequence[int] = range(5), max_iters: int = 1 << 20):
    t, D = _i32(tour).copy(), _i32(D)
    nbs_a = _i32(sorted(nbs))
    fc, ev, mv = C.c_int64(), C.c_int64(), C.c_int64()
    it = lib().orc_dvnd_total(len(t), _p(t), D.shape[0], _p(D), int(wide), len(nbs_a), _p(nbs_a), max_iters,
                              C.byref(fc), C.byref(ev), C.byref(mv))
    return t, {"cost": fc.value, "iterations": it, "evals": ev.value, "moves": mv.value}


def sweep(tour, D, wide: bool = False, nbs: Sequence[int] = range(5), threads: int = 1):
    t, D = _i32(tour), _i32(D)
    nbs_a = _i32(list(nbs))
    tot = sum(num_blocks(nb, len(t)) for nb in nbs)
    c = np.zeros(tot, np.int64)
    i = np.zeros(tot, np.int32)
    j = np.zeros(tot, np.int32)
    ev = lib().orc_sweep(len(t), _p(t), D.shape[0], _p(D), int(wide), len(nbs_a), _p(nbs_a), threads, _p(c), _p(i),
                         _p(j))
    return int(ev), c, i, j


def legacy_no_conflict(m1, m2) -> bool:
    return bool(lib().orc_legacy_no_conflict(m1[0], m1[1], m1[2], m2[0], m2[1], m2[2]))


def legacy_better_no_conflict(moves, maximize: bool = False, melhor_para_pior: bool = False):
    m = len(moves)
    ids = _i32([mv[0] for mv in moves])
    is_ = _i32([mv[1] for mv in moves])
    js = _i32([mv[2] for mv in moves])
    cs = _i32([mv[3] for mv in moves])
    sel = np.zeros(max(m, 1), np.int32)
    imp = np.zeros(1, np.int32)
    k = lib().orc_legacy_better_no_conflict(m, _p(ids), _p(is_), _p(js), _p(cs), _p(sel), _p(imp), int(maximize),
                                            int(melhor_para_pior))
    return sel[:k].tolist(), int(imp[0]), k


def legacy_apply_moves(tour, D, moves):
    t, D = _i32(tour).copy(), _i32(D)
    ids = _i32([mv[0] for mv in moves])
    is_ = _i32([mv[1] for mv in moves])
    js = _i32([mv[2] for mv in moves])
    c = lib().orc_legacy_apply_moves(len(t), _p(t), D.shape[0], _p(D), len(moves), _p(ids), _p(is_), _p(js))
    return t, int(c)


# ---------------------------------------------------------------- generators
# The benchmark's seeded generators live in the product package (pure numpy,
# no GPU); they are re-exported here so tests can build the same inputs.
import sys as _sys  # noqa: E402

_sys.path.insert(0, os.path.join(os.path.dirname(HERE), "wamca-gpu-mi_gb300"))
from mlpgpu.workloads import (clustered_instance, log_uniform_sizes, random_perm_tour,  # noqa: E402,F401
                              uniform_instance)
