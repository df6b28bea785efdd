"""Python host binding of libmlpgpu.so (the GB300 MLP local-search engine).

A thin ctypes layer over the C-ABI of include/mlp_gpu.h and
include/wamca_dvnd.h, shaped like the reference's task API:

    MLProblem  -> Problem   (source/mlproblem.h:61-151)
    MLSolution + MLKernel{Swap,2Opt,OrOpt}
               -> Solver    (source/mlsolution.h:62-434, source/mlkernel.h:104-318)
    legacy extern "C" DVND entry points -> Legacy (source/dvnd.cuh, source/dvnd.h)

There is no CPU fallback: every call goes to the CUDA library, and importing
this module fails loudly if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libmlpgpu.so")
TUNING_PATH = os.path.join(_HERE, "tuning_gb300.json")

NB_SWAP, NB_2OPT, NB_OROPT1, NB_OROPT2, NB_OROPT3 = range(5)
NB_ALL = 0x1F
# Compiled sweep tile shapes (diagonals x rows; the last four give the DVND
# sweep two diagonals per thread), indices 0 .. NUM_TILE_SHAPES - 1.
TILE_SHAPES = ((32, 4), (32, 8), (32, 16), (64, 4), (64, 8), (64, 16), (128, 8), (128, 16), (32, 32), (64, 32),
               (64, 8), (64, 16), (64, 32), (128, 16))
NUM_TILE_SHAPES = len(TILE_SHAPES)
NB_NAMES = ("swap", "2opt", "oropt1", "oropt2", "oropt3")


class MLPError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class DvndStats(C.Structure):
    _fields_ = [
        ("cost", C.c_int64),
        ("iterations", C.c_int64),
        ("sweeps", C.c_int64),
        ("moves", C.c_int64),
        ("evals", C.c_int64),
        ("converged", C.c_int32),
        ("reserved", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_ if f != "reserved"}


class ServeInfo(C.Structure):
    _fields_ = [
        ("arrival", C.c_double),
        ("admitted", C.c_double),
        ("finished", C.c_double),
        ("status", C.c_int32),
        ("n", C.c_int32),
    ]


PENDING = 10
CANCELLED = 9


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Loads libmlpgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                          "or python wamca-gpu-mi_gb300/build_lib.py")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, u32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32
    P = C.POINTER
    sig = {
        "mlp_version": (C.c_int, []),
        "mlp_last_error": (C.c_char_p, []),
        "mlp_status_string": (C.c_char_p, [C.c_int]),
        "mlp_device_count": (C.c_int, [P(i32)]),
        "mlp_set_device": (C.c_int, [i32]),
        "mlp_problem_create_coords": (C.c_int, [i32, vp, vp, i32, i32, P(vp)]),
        "mlp_problem_create_coords_device": (C.c_int, [i32, vp, vp, i32, i32, P(vp)]),
        "mlp_problem_create_matrix": (C.c_int, [i32, vp, i32, P(vp)]),
        "mlp_problem_load_tsplib": (C.c_int, [C.c_char_p, i32, i32, P(vp)]),
        "mlp_problem_info": (C.c_int, [vp, P(i32), P(i32), P(i32)]),
        "mlp_problem_get_dist": (C.c_int, [vp, vp]),
        "mlp_problem_destroy": (None, [vp]),
        "mlp_solver_create": (C.c_int, [vp, i32, P(vp)]),
        "mlp_solver_destroy": (None, [vp]),
        "mlp_solver_set_stream": (C.c_int, [vp, vp]),
        "mlp_solver_set_tile_shape": (C.c_int, [vp, i32]),
        "mlp_solver_set_unroll": (C.c_int, [vp, i32]),
        "mlp_solver_set_sweep_kernel": (C.c_int, [vp, i32]),
        "mlp_solver_set_merge_mode": (C.c_int, [vp, i32]),
        "mlp_solver_set_total": (C.c_int, [vp, i32]),
        "mlp_solver_eval_oropt": (C.c_int, [vp, i32, vp, vp, vp]),
        "mlp_solver_pass_oropt": (C.c_int, [vp, i32, i32, vp, vp, vp, P(i32), P(i64)]),
        "mlp_solver_set_tour": (C.c_int, [vp, vp, i32]),
        "mlp_solver_set_tour_device": (C.c_int, [vp, vp, i32]),
        "mlp_solver_get_tour": (C.c_int, [vp, vp, i32]),
        "mlp_solver_save": (C.c_int, [vp, C.c_char_p]),
        "mlp_solver_load": (C.c_int, [vp, C.c_char_p]),
        "mlp_solver_tour_device": (C.c_int, [vp, P(vp)]),
        "mlp_solver_cost": (C.c_int, [vp, P(i64)]),
        "mlp_solver_weights": (C.c_int, [vp, vp, i32]),
        "mlp_solver_ads": (C.c_int, [vp, vp, i64]),
        "mlp_solver_num_candidates": (C.c_int, [vp, i32, P(i32)]),
        "mlp_solver_eval": (C.c_int, [vp, i32, vp, vp, vp]),
        "mlp_solver_pass": (C.c_int, [vp, i32, i32, vp, vp, vp, vp, P(i32), P(i64)]),
        "mlp_solver_dvnd": (C.c_int, [vp, i32, i32, P(DvndStats)]),
        "mlp_solver_begin": (C.c_int, [vp, i32, i32]),
        "mlp_solver_dvnd_async": (C.c_int, [vp, i32, i32]),
        "mlp_batch_run_async": (C.c_int, [vp, i32, i32]),
        "mlp_solver_enqueue": (C.c_int, [vp, i32]),
        "mlp_solver_stats": (C.c_int, [vp, P(DvndStats)]),
        "mlp_solver_sweep": (C.c_int, [vp, i32, i32, P(i64)]),
        "mlp_solver_autotune": (C.c_int, [vp, P(i32)]),
        "mlp_solver_time_sweep": (C.c_int, [vp, i32, i32, vp, C.c_int64, P(C.c_float)]),
        "mlp_eval_noalloc": (C.c_int, [vp, i32, vp, i32, i32, vp, vp, vp, vp]),
        "mlp_tuning_set": (C.c_int, [vp, vp, vp, i32]),
        "mlp_tuning_get": (C.c_int, [vp, vp, vp, i32, P(i32)]),
        "mlp_tuning_load": (C.c_int, [C.c_char_p]),
        "mlp_batch_create": (C.c_int, [i32, P(vp)]),
        "mlp_batch_destroy": (None, [vp]),
        "mlp_batch_set_stream": (C.c_int, [vp, vp]),
        "mlp_batch_set_tile_shape": (C.c_int, [vp, i32]),
        "mlp_batch_set_merge_mode": (C.c_int, [vp, i32]),
        "mlp_batch_set_sweep_kernel": (C.c_int, [vp, i32]),
        "mlp_batch_set_total": (C.c_int, [vp, i32]),
        "mlp_batch_set_check_interval": (C.c_int, [vp, i32]),
        "mlp_batch_add": (C.c_int, [vp, vp, vp, i32, P(i32)]),
        "mlp_batch_add_random": (C.c_int, [vp, vp, C.c_uint32, C.c_float, P(i32)]),
        "mlp_batch_add_random_ties": (C.c_int, [vp, vp, C.c_uint32, C.c_float, i32, P(i32)]),
        "mlp_solver_random_tour": (C.c_int, [vp, C.c_uint32, C.c_float]),
        "mlp_solver_random_tour_ties": (C.c_int, [vp, C.c_uint32, C.c_float, i32]),
        "mlp_problem_random_tours": (C.c_int, [vp, i32, vp, C.c_float, vp]),
        "mlp_problem_random_tours_ties": (C.c_int, [vp, i32, vp, C.c_float, i32, vp]),
        "mlp_batch_run": (C.c_int, [vp, i32, i32]),
        "mlp_batch_reset": (C.c_int, [vp]),
        "mlp_batch_result": (C.c_int, [vp, i32, vp, i32, P(DvndStats)]),
        "mlp_server_create": (C.c_int, [i64, i32, i32, P(vp)]),
        "mlp_server_destroy": (None, [vp]),
        "mlp_server_now": (C.c_double, [vp]),
        "mlp_server_footprint": (i64, [i32, i32]),
        "mlp_server_set_tile_shape": (C.c_int, [vp, i32]),
        "mlp_server_submit": (C.c_int, [vp, i32, vp, vp, i32, vp, i32, i32, i32, C.c_double, P(i64)]),
        "mlp_server_step": (C.c_int, [vp, i32, P(i32), P(i32)]),
        "mlp_server_finished": (C.c_int, [vp, P(i64), i32, P(i32)]),
        "mlp_server_result": (C.c_int, [vp, i64, vp, i32, P(DvndStats), P(ServeInfo)]),
        "mlp_server_cancel": (C.c_int, [vp, i64]),
        "mlp_server_status": (C.c_int, [vp, P(i64), P(i32), P(i32), P(i32)]),
        "mlp_server_fail_next_admissions": (C.c_int, [vp, i32]),
        "bestNeighborSimple": (C.c_uint, [C.c_char_p, vp, C.c_uint, C.c_int]),
        "bestNeighbor": (C.c_uint, [C.c_char_p, vp, C.c_uint, C.c_int, C.c_bool, C.c_uint, vp, vp, vp,
                                    vp, vp, C.c_bool, C.c_uint, vp]),
        "applyMoves": (C.c_uint, [C.c_char_p, vp, C.c_uint, C.c_uint, vp, vp, vp, vp]),
        "getNoConflictMoves": (C.c_int, [C.c_uint, vp, vp, vp, vp, vp, vp, C.c_bool, C.c_bool]),
        "noConflict": (C.c_bool, [C.c_ushort, C.c_uint, C.c_uint, C.c_ushort, C.c_uint, C.c_uint]),
        "segFault": (None, []),
        "mlp_legacy_reset": (None, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    # The tile-shape table the autotuner measured on GB300 (shapes only: results
    # never depend on it).
    if os.path.exists(TUNING_PATH):
        L.mlp_tuning_load(TUNING_PATH.encode())
    return L


def tuning_table() -> list:
    """Current tile-shape table: [(max tour size, shape for one job, shape for many jobs), ...]."""
    a, b, c = (np.zeros(64, np.int32) for _ in range(3))
    k = C.c_int32()
    _check(lib().mlp_tuning_get(_ptr(a), _ptr(b), _ptr(c), 64, C.byref(k)))
    return [(int(a[q]), int(b[q]), int(c[q])) for q in range(k.value)]


def set_tuning_table(rows) -> None:
    """Sets the tile-shape table from (max tour size, shape one, shape many) rows ([] clears it)."""
    a = np.array([r[0] for r in rows], np.int32)
    b = np.array([r[1] for r in rows], np.int32)
    c = np.array([r[2] for r in rows], np.int32)
    _check(lib().mlp_tuning_set(_ptr(a), _ptr(b), _ptr(c), len(rows)))


def _check(status: int) -> None:
    if status != 0:
        raise MLPError(status, lib().mlp_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def device_count() -> int:
    c = C.c_int32(0)
    st = lib().mlp_device_count(C.byref(c))
    return c.value if st == 0 else 0


class Problem:
    """MLProblem: an instance resident on the GPU (n x n int32 distances)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        n, size, dmax = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().mlp_problem_info(self._h, C.byref(n), C.byref(size), C.byref(dmax)))
        self.n, self.size, self.max_dist = n.value, size.value, dmax.value

    @classmethod
    def from_coords(cls, x: Sequence[int], y: Sequence[int], dist_round: bool = True,
                    cost_tour: bool = True) -> "Problem":
        x, y = _i32(x), _i32(y)
        h = C.c_void_p()
        _check(lib().mlp_problem_create_coords(len(x), _ptr(x), _ptr(y), int(cost_tour),
                                               int(dist_round), C.byref(h)))
        return cls(h)

    @classmethod
    def from_coords_device(cls, n: int, x_dev: int, y_dev: int, dist_round: bool = True) -> "Problem":
        h = C.c_void_p()
        _check(lib().mlp_problem_create_coords_device(n, C.c_void_p(x_dev), C.c_void_p(y_dev), 1,
                                                      int(dist_round), C.byref(h)))
        return cls(h)

    @classmethod
    def from_matrix(cls, D: np.ndarray, cost_tour: bool = True) -> "Problem":
        D = _i32(D)
        h = C.c_void_p()
        _check(lib().mlp_problem_create_matrix(D.shape[0], _ptr(D), int(cost_tour), C.byref(h)))
        return cls(h)

    @classmethod
    def load_tsplib(cls, path: str, dist_round: bool = False, cost_tour: bool = True) -> "Problem":
        h = C.c_void_p()
        _check(lib().mlp_problem_load_tsplib(path.encode(), int(cost_tour), int(dist_round), C.byref(h)))
        return cls(h)

    def dist(self) -> np.ndarray:
        D = np.zeros((self.n, self.n), np.int32)
        _check(lib().mlp_problem_get_dist(self._h, _ptr(D)))
        return D

    def random_tours(self, seeds: Sequence[int], alpha: float = 0.5, ties: int = 0) -> np.ndarray:
        """Starts of MLSolution::random(seed, alpha) built on the device, one row
        per seed; equal distances in client-id order (ties=0) or in the
        reference's own std::sort order (ties=1)."""
        sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint32))
        out = np.zeros((len(sd), self.n + 1), np.int32)
        _check(lib().mlp_problem_random_tours_ties(self._h, len(sd), _ptr(sd), C.c_float(alpha), int(ties),
                                                   _ptr(out)))
        return out

    def close(self) -> None:
        if self._h:
            lib().mlp_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """MLSolution + the MLKernel tasks of one instance (device-resident state)."""

    def __init__(self, problem: Problem, wide: bool = False):
        self.problem = problem
        self.wide = bool(wide)
        self._h = C.c_void_p()
        _check(lib().mlp_solver_create(problem._h, int(wide), C.byref(self._h)))
        self.size = problem.size

    def close(self) -> None:
        if self._h:
            lib().mlp_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int) -> None:
        _check(lib().mlp_solver_set_stream(self._h, C.c_void_p(stream_handle)))

    def set_tile_shape(self, shape: int) -> None:
        _check(lib().mlp_solver_set_tile_shape(self._h, shape))

    def set_unroll(self, u: int) -> None:
        """Loop mode of dvnd(): 0 (default) the device-side loop (a CUDA-graph
        while node, 16 iterations a pass); u >= 1 replays graphs of u
        iterations and checks convergence on the host in between."""
        _check(lib().mlp_solver_set_unroll(self._h, u))

    def set_sweep_kernel(self, variant: int) -> None:
        """DVND sweep kernel: 1 (default) row/column term tables, 0 the
        general fused sweep; identical results."""
        _check(lib().mlp_solver_set_sweep_kernel(self._h, variant))

    def set_merge_mode(self, mode: int) -> None:
        """0 automatic, 1 six-CTA cluster, 2 one CTA; identical results."""
        _check(lib().mlp_solver_set_merge_mode(self._h, mode))

    def set_total(self, on: bool = True) -> None:
        """TOTAL multi-improvement (MLKernel isTotal): every evaluated move is a
        merge candidate, not only each reference block's best."""
        _check(lib().mlp_solver_set_total(self._h, int(bool(on))))

    def set_tour(self, tour: Sequence[int]) -> None:
        t = _i32(tour)
        _check(lib().mlp_solver_set_tour(self._h, _ptr(t), len(t)))

    def random_tour(self, seed: int, alpha: float = 0.5, ties: int = 0) -> None:
        """The tour becomes MLSolution::random(seed, alpha), built on the device
        (ties as in Problem.random_tours)."""
        _check(lib().mlp_solver_random_tour_ties(self._h, seed, C.c_float(alpha), int(ties)))

    def set_tour_device(self, ptr: int) -> None:
        _check(lib().mlp_solver_set_tour_device(self._h, C.c_void_p(ptr), self.size))

    def save(self, path: str) -> None:
        """Writes the current tour and cost in MLSolution's text format."""
        _check(lib().mlp_solver_save(self._h, path.encode()))

    def load(self, path: str) -> None:
        """Resumes from a tour saved in MLSolution's text format (cost recomputed)."""
        _check(lib().mlp_solver_load(self._h, path.encode()))

    def tour(self) -> np.ndarray:
        t = np.zeros(self.size, np.int32)
        _check(lib().mlp_solver_get_tour(self._h, _ptr(t), self.size))
        return t

    def tour_device_ptr(self) -> int:
        p = C.c_void_p()
        _check(lib().mlp_solver_tour_device(self._h, C.byref(p)))
        return p.value

    def cost(self) -> int:
        c = C.c_int64()
        _check(lib().mlp_solver_cost(self._h, C.byref(c)))
        return c.value

    def weights(self) -> np.ndarray:
        w = np.zeros(self.size, np.int32)
        _check(lib().mlp_solver_weights(self._h, _ptr(w), self.size))
        return w

    def ads(self) -> np.ndarray:
        words = 32 + self.size * (self.size + 3)
        a = np.zeros(words, np.uint32)
        _check(lib().mlp_solver_ads(self._h, _ptr(a), words))
        return a

    def num_candidates(self, nb: int) -> int:
        c = C.c_int32()
        _check(lib().mlp_solver_num_candidates(self._h, nb, C.byref(c)))
        return c.value

    def eval(self, nb: int):
        m = self.num_candidates(nb)
        cost = np.zeros(m, np.int64)
        i = np.zeros(m, np.int32)
        j = np.zeros(m, np.int32)
        _check(lib().mlp_solver_eval(self._h, nb, _ptr(cost), _ptr(i), _ptr(j)))
        return cost, i, j

    def pass_(self, nb: int, max_moves: int = 1 << 15):
        ids = np.zeros(max_moves, np.int32)
        i = np.zeros(max_moves, np.int32)
        j = np.zeros(max_moves, np.int32)
        c = np.zeros(max_moves, np.int64)
        cnt, nc = C.c_int32(), C.c_int64()
        _check(lib().mlp_solver_pass(self._h, nb, max_moves, _ptr(ids), _ptr(i), _ptr(j), _ptr(c),
                                     C.byref(cnt), C.byref(nc)))
        k = min(cnt.value, max_moves)
        return nc.value, list(zip(ids[:k].tolist(), i[:k].tolist(), j[:k].tolist(), c[:k].tolist()))

    def eval_oropt(self, k: int):
        """Per-block candidates of Or-opt-k (k in [1, 28])."""
        m = self.size - k - 2
        cost = np.zeros(max(m, 0), np.int64)
        i = np.zeros(max(m, 0), np.int32)
        j = np.zeros(max(m, 0), np.int32)
        _check(lib().mlp_solver_eval_oropt(self._h, k, _ptr(cost), _ptr(i), _ptr(j)))
        return cost, i, j

    def pass_oropt(self, k: int, max_moves: int = 1 << 15):
        """One Or-opt-k pass; returns (new cost, [(id, i, j, cost)]) with id = k + 1."""
        i = np.zeros(max_moves, np.int32)
        j = np.zeros(max_moves, np.int32)
        c = np.zeros(max_moves, np.int64)
        cnt, nc = C.c_int32(), C.c_int64()
        _check(lib().mlp_solver_pass_oropt(self._h, k, max_moves, _ptr(i), _ptr(j), _ptr(c), C.byref(cnt),
                                           C.byref(nc)))
        n = min(cnt.value, max_moves)
        return nc.value, [(k + 1, a, b, d) for a, b, d in zip(i[:n].tolist(), j[:n].tolist(), c[:n].tolist())]

    def dvnd(self, nb_mask: int = NB_ALL, max_iters: int = 1 << 20) -> dict:
        st = DvndStats()
        _check(lib().mlp_solver_dvnd(self._h, nb_mask, max_iters, C.byref(st)))
        return st.as_dict()

    def dvnd_async(self, nb_mask: int = NB_ALL, max_iters: int = 1 << 20) -> None:
        _check(lib().mlp_solver_dvnd_async(self._h, nb_mask, max_iters))

    def begin(self, nb_mask: int = NB_ALL, max_iters: int = 1 << 20) -> None:
        _check(lib().mlp_solver_begin(self._h, nb_mask, max_iters))

    def enqueue(self, iterations: int) -> None:
        _check(lib().mlp_solver_enqueue(self._h, iterations))

    def stats(self) -> dict:
        st = DvndStats()
        _check(lib().mlp_solver_stats(self._h, C.byref(st)))
        return st.as_dict()

    def sweep(self, nb_mask: int = NB_ALL, repeats: int = 1) -> int:
        e = C.c_int64()
        _check(lib().mlp_solver_sweep(self._h, nb_mask, repeats, C.byref(e)))
        return e.value

    def autotune(self) -> int:
        s = C.c_int32()
        _check(lib().mlp_solver_autotune(self._h, C.byref(s)))
        return s.value

    def time_sweep(self, nb_mask: int = NB_ALL, repeats: int = 20, flush_ptr: int = 0, flush_bytes: int = 0) -> float:
        """Time (seconds) of one launch of the solver's sweep kernel, by CUDA
        events on the solver's stream (mlp_solver_time_sweep): warm, the mean
        of `repeats` back-to-back launches; with a flush buffer (device pointer
        and size), overwritten before every launch, the median of launches
        that each start cold."""
        ms = C.c_float()
        _check(lib().mlp_solver_time_sweep(self._h, nb_mask, repeats, C.c_void_p(flush_ptr or None), flush_bytes,
                                           C.byref(ms)))
        return ms.value * 1e-3


def eval_noalloc(dist_dev: int, n: int, tour_dev: int, nb: int, wide: bool, cost_dev: int, i_dev: int,
                 j_dev: int, stream: int = 0) -> None:
    """mlp_eval_noalloc: per-block candidates of neighbourhood nb computed
    from caller-owned device buffers, without any allocation."""
    _check(lib().mlp_eval_noalloc(C.c_void_p(dist_dev), n, C.c_void_p(tour_dev), nb, int(wide),
                                  C.c_void_p(cost_dev), C.c_void_p(i_dev), C.c_void_p(j_dev),
                                  C.c_void_p(stream)))


class Batch:
    """Batched form: many DVND searches advanced by the same launches."""

    def __init__(self, wide: bool = False):
        self._h = C.c_void_p()
        _check(lib().mlp_batch_create(int(wide), C.byref(self._h)))
        self.sizes: list[int] = []
        self._problems: list[Problem] = []

    def close(self) -> None:
        if self._h:
            lib().mlp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int) -> None:
        _check(lib().mlp_batch_set_stream(self._h, C.c_void_p(stream_handle)))

    def set_tile_shape(self, shape: int) -> None:
        _check(lib().mlp_batch_set_tile_shape(self._h, shape))

    def set_merge_mode(self, mode: int) -> None:
        """0 automatic, 1 six-CTA cluster per job, 2 one CTA per job."""
        _check(lib().mlp_batch_set_merge_mode(self._h, mode))

    def set_sweep_kernel(self, variant: int) -> None:
        """DVND sweep kernel of the batch (as Solver.set_sweep_kernel)."""
        _check(lib().mlp_batch_set_sweep_kernel(self._h, variant))

    def set_total(self, on: bool = True) -> None:
        """TOTAL candidate mode for every search of the batch (as Solver.set_total)."""
        _check(lib().mlp_batch_set_total(self._h, int(bool(on))))

    def set_check_interval(self, iterations: int) -> None:
        """Iterations between convergence checks (converged jobs then leave the launches)."""
        _check(lib().mlp_batch_set_check_interval(self._h, iterations))

    def add(self, problem: Problem, tour: Sequence[int]) -> int:
        t = _i32(tour)
        j = C.c_int32()
        _check(lib().mlp_batch_add(self._h, problem._h, _ptr(t), len(t), C.byref(j)))
        self.sizes.append(len(t))
        self._problems.append(problem)
        return j.value

    def add_random(self, problem: Problem, seed: int, alpha: float = 0.5, ties: int = 0) -> int:
        """Adds a search whose start MLSolution::random(seed, alpha) is built on
        the device (ties as in Problem.random_tours)."""
        j = C.c_int32()
        _check(lib().mlp_batch_add_random_ties(self._h, problem._h, seed, C.c_float(alpha), int(ties), C.byref(j)))
        self.sizes.append(problem.n + 1)
        self._problems.append(problem)
        return j.value

    def run(self, nb_mask: int = NB_ALL, max_iters: int = 1 << 20) -> None:
        _check(lib().mlp_batch_run(self._h, nb_mask, max_iters))

    def run_async(self, nb_mask: int = NB_ALL, max_iters: int = 1 << 20) -> None:
        _check(lib().mlp_batch_run_async(self._h, nb_mask, max_iters))

    def reset(self) -> None:
        _check(lib().mlp_batch_reset(self._h))

    def result(self, job: int):
        t = np.zeros(self.sizes[job], np.int32)
        st = DvndStats()
        _check(lib().mlp_batch_result(self._h, job, _ptr(t), len(t), C.byref(st)))
        return t, st.as_dict()


def save_solution(path: str, tour: Sequence[int], cost: int) -> None:
    """Checkpoints a result (e.g. of a served or batched search) in the text
    format of the reference's MLSolution::save: tour length, cost, tour."""
    t = [int(v) for v in tour]
    with open(path, "w") as f:
        f.write(f"{len(t)}\n{int(cost)}\n{' '.join(str(v) for v in t)}\n")


def load_solution(path: str):
    """Reads a tour saved by save_solution / mlp_solver_save / MLSolution::save;
    returns (tour, stored cost).  Re-submit the tour to resume the search."""
    with open(path) as f:
        vals = f.read().split()
    if len(vals) < 2:
        raise ValueError("invalid solution file: missing length or cost")
    size, cost = int(vals[0]), int(vals[1])
    tour = np.array([int(v) for v in vals[2:2 + size]], dtype=np.int32)
    if len(tour) != size:
        raise ValueError("invalid solution file: truncated tour")
    return tour, cost


class Server:
    """Serving form: continuous batching of DVND searches that arrive over time.

    submit() queues a search; step() admits queued searches while slots and the
    memory budget allow, runs `iters` DVND iterations over every admitted search
    in shared launches and retires the finished ones; finished() lists the ids
    that completed and result() takes one result.
    """

    def __init__(self, memory_budget: int, wide: bool = False, max_active: int = 512):
        self._h = C.c_void_p()
        _check(lib().mlp_server_create(int(memory_budget), int(wide), int(max_active), C.byref(self._h)))
        self.wide = wide

    def close(self) -> None:
        if self._h:
            lib().mlp_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def footprint(n: int, wide: bool = False) -> int:
        return int(lib().mlp_server_footprint(n, int(wide)))

    def now(self) -> float:
        return float(lib().mlp_server_now(self._h))

    def set_tile_shape(self, shape: int) -> None:
        _check(lib().mlp_server_set_tile_shape(self._h, shape))

    def submit(self, x, y, tour, dist_round: bool = True, nb_mask: int = NB_ALL, max_iters: int = 1 << 20,
               arrival: float = -1.0) -> int:
        x, y, t = _i32(x), _i32(y), _i32(tour)
        rid = C.c_int64()
        _check(lib().mlp_server_submit(self._h, len(x), _ptr(x), _ptr(y), int(dist_round), _ptr(t), len(t),
                                       nb_mask, max_iters, float(arrival), C.byref(rid)))
        return rid.value

    def step(self, iters: int = 1):
        a, q = C.c_int32(), C.c_int32()
        _check(lib().mlp_server_step(self._h, iters, C.byref(a), C.byref(q)))
        return a.value, q.value

    def finished(self, cap: int = 4096) -> list:
        ids = (C.c_int64 * cap)()
        k = C.c_int32()
        _check(lib().mlp_server_finished(self._h, ids, cap, C.byref(k)))
        return [int(ids[i]) for i in range(k.value)]

    def result(self, rid: int, n: int):
        """(tour, stats, info) of a finished request, or None while pending."""
        t = np.zeros(n + 1, np.int32)
        st, info = DvndStats(), ServeInfo()
        s = lib().mlp_server_result(self._h, rid, _ptr(t), len(t), C.byref(st), C.byref(info))
        if s == PENDING:
            return None
        _check(s)
        return t, st.as_dict(), {f: getattr(info, f) for f, _ in info._fields_}

    def cancel(self, rid: int) -> None:
        _check(lib().mlp_server_cancel(self._h, rid))

    def status(self) -> dict:
        m, a, q, f = C.c_int64(), C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().mlp_server_status(self._h, C.byref(m), C.byref(a), C.byref(q), C.byref(f)))
        return {"mem_in_use": m.value, "active": a.value, "queued": q.value, "finished": f.value}

    def fail_next_admissions(self, count: int) -> None:
        _check(lib().mlp_server_fail_next_admissions(self._h, count))


class Legacy:
    """The reference's extern "C" DVND entry points (include/wamca_dvnd.h)."""

    @staticmethod
    def best_neighbor(file: str, solution: np.ndarray, nb: int, just_calc: bool = False,
                      host_code: int = 0, use_moves: int = 0, solution_resp: Optional[np.ndarray] = None):
        sol = solution
        um = C.c_uint(use_moves)
        cap = max(use_moves, 1)
        ids = np.zeros(cap, np.uint16)
        is_ = np.zeros(cap, np.uint32)
        js = np.zeros(cap, np.uint32)
        cs = np.zeros(cap, np.int32)
        resp_ptr = _ptr(solution_resp) if solution_resp is not None else None
        r = lib().bestNeighbor(file.encode(), _ptr(sol), len(sol), nb, just_calc, host_code, C.byref(um),
                               _ptr(ids), _ptr(is_), _ptr(js), _ptr(cs), False, 1, resp_ptr)
        k = um.value if use_moves else 0
        return r, list(zip(ids[:k].tolist(), is_[:k].tolist(), js[:k].tolist(), cs[:k].tolist()))

    @staticmethod
    def apply_moves(file: str, solution: np.ndarray, moves) -> int:
        m = len(moves)
        ids = np.array([mv[0] for mv in moves], np.uint16)
        is_ = np.array([mv[1] for mv in moves], np.uint32)
        js = np.array([mv[2] for mv in moves], np.uint32)
        cs = np.array([mv[3] if len(mv) > 3 else 0 for mv in moves], np.int32)
        return lib().applyMoves(file.encode(), _ptr(solution), len(solution), m, _ptr(ids), _ptr(is_),
                                _ptr(js), _ptr(cs))

    @staticmethod
    def no_conflict_moves(moves, maximize: bool = False, melhor_para_pior: bool = False):
        m = len(moves)
        ids = np.array([mv[0] for mv in moves], np.uint16)
        is_ = np.array([mv[1] for mv in moves], np.uint32)
        js = np.array([mv[2] for mv in moves], np.uint32)
        cs = np.array([mv[3] for mv in moves], np.int32)
        sel = np.zeros(max(m, 1), np.int32)
        imp = np.zeros(1, np.int32)
        k = lib().getNoConflictMoves(m, _ptr(ids), _ptr(is_), _ptr(js), _ptr(cs), _ptr(sel), _ptr(imp),
                                     maximize, melhor_para_pior)
        return sel[:max(k, 0)].tolist(), int(imp[0]), k

    @staticmethod
    def no_conflict(id1, i1, j1, id2, i2, j2) -> bool:
        return bool(lib().noConflict(id1, i1, j1, id2, i2, j2))

    @staticmethod
    def reset() -> None:
        lib().mlp_legacy_reset()
