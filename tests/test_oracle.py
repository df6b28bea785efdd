"""CPU tests of the oracle (the checker) against the reference's known answers
and the golden fixtures generated from the reference's compiled evaluator."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN


@pytest.fixture(scope="module")
def berlin():
    with open(os.path.join(GOLDEN, "berlin52.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def cases():
    with open(os.path.join(GOLDEN, "ref_cases.json")) as f:
        return json.load(f)


def test_k1_mtrand(berlin):
    # tests/mtrand.Test.cpp:11-48
    assert oracle.mt_rand(0, 5).tolist() == [2357136044, 2546248239, 3071714933, 3626093760, 2588848963]
    assert (oracle.mt_rand(0, 6) % 10).tolist() == [4, 9, 3, 0, 3, 9]
    assert (oracle.mt_rand(1, 5) % 10).tolist() == [5, 9, 4, 8, 3]
    for mx, vals in berlin["mt_rand_max_seed12345"].items():
        assert oracle.mt_rand_max(12345, int(mx), 16).tolist() == vals


def test_k2_k3_berlin52(berlin):
    # tests/mlproblem.Test.cpp:11-28 (size 53) and tests/mlsolution.Test.cpp:62-80 (494309)
    x, y = np.array(berlin["x"], np.int32), np.array(berlin["y"], np.int32)
    assert len(x) + 1 == berlin["size"] == 53
    D = oracle.dist(x, y, False)
    t = oracle.random_tour(D, 0, 0.5)
    assert t.tolist() == berlin["random_tour_seed0"]
    assert oracle.cost(t, D) == berlin["cost_random_tour_seed0"] == 494309


def test_k4_swap_pass(berlin):
    # tests/WamcaExperiment.Test.cpp:70-131
    x, y = np.array(berlin["x"], np.int32), np.array(berlin["y"], np.int32)
    D = oracle.dist(x, y, False)
    t = np.array(berlin["random_tour_seed0"], np.int32)
    nt, c, moves = oracle.pass_(0, t, D)
    assert c == berlin["k4_cost_after_swap_pass"] == 367403
    assert len(moves) == 6
    assert c == oracle.cost(nt, D)


def test_ads_matches_reference_ldsupdate(berlin):
    x, y = np.array(berlin["x"], np.int32), np.array(berlin["y"], np.int32)
    D = oracle.dist(x, y, False)
    t = np.array(berlin["random_tour_seed0"], np.int32)
    a = oracle.ads(t, D, x, y, False)
    ref = np.array(berlin["ads_random_tour_seed0"], np.uint32)
    assert np.array_equal(a[:6], ref[:6]) and np.array_equal(a[32:], ref[32:])


def test_reference_cases(cases):
    for c in cases:
        x, y = np.array(c["x"], np.int32), np.array(c["y"], np.int32)
        D = oracle.dist(x, y, bool(c["dist_round"]))
        t = oracle.random_tour(D, c["seed"], 0.5)
        assert t.tolist() == c["tour"], c["instance"]
        assert oracle.cost(t, D) == c["cost"], c["instance"]
        a = oracle.ads(t, D, x, y, bool(c["dist_round"]))
        h = hashlib.sha256()
        h.update(a[:6].astype("<u4").tobytes())
        h.update(a[32:].astype("<u4").tobytes())
        assert h.hexdigest() == c["ads_sha256"], c["instance"]


@pytest.mark.parametrize("n,seed,rnd", [(5, 1, True), (6, 2, False), (9, 3, True), (31, 4, True), (52, 5, False)])
def test_deltas_faithful_fast_bruteforce(n, seed, rnd):
    x, y = oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, rnd)
    t = oracle.random_perm_tour(n, seed)
    size = n + 1
    for nb in range(5):
        f = oracle.eval_nb(nb, t, D, faithful=True)
        q = oracle.eval_nb(nb, t, D, faithful=False)
        for a, b in zip(f, q):
            assert np.array_equal(a, b)
    # exhaustive brute force on all moves of every neighbourhood
    for i in range(1, size - 1):
        for j in range(1, size - 1):
            for mid in range(5):
                k = mid - 1
                if mid == 0 and not (j >= i + 2 and j <= size - 2):
                    continue
                if mid == 1 and not (j >= i + 1 and j <= size - 2):
                    continue
                if mid >= 2 and not ((i < j and j + k <= size - 1) or (i > j + 1 and i + k <= size - 1)):
                    continue
                assert oracle.move_delta(mid, i, j, t, D) == oracle.move_delta(mid, i, j, t, D, brute=True)


def test_int32_wraparound_matches_int64_mod_2_32():
    n = 400
    x, y = oracle.uniform_instance(n, 9, box=20000)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 9)
    assert oracle.cost(t, D, wide=False) == oracle.cost(t, D, wide=True) % (1 << 32)


def test_merge_predicates_imply_disjoint_footprints():
    """Every pair canMerge accepts touches disjoint tour positions, so the
    selected moves can be applied in any order (and in parallel)."""
    size = 16
    moves = []
    for i in range(1, size - 1):
        moves += [(0, i, j) for j in range(i + 2, size - 1)]
        moves += [(1, i, j) for j in range(i + 1, size - 1)]
    for k in (1, 2, 3):
        for i in range(1, size - 1):
            for j in range(1, size - 1):
                if (i < j and j + k <= size - 1) or (i > j + 1 and i + k <= size - 1):
                    moves.append((k + 1, i, j))

    def fp(m):
        mid, i, j = m
        if mid == 0:
            return {i, j}
        if mid == 1:
            return set(range(i, j + 1))
        k = mid - 1
        return set(range(i, j + k)) if i < j else set(range(j, i + k))

    for a in moves:
        fa = fp(a)
        for b in moves:
            if oracle.can_merge(a, b):
                assert not (fa & fp(b)), (a, b)


def test_dvnd_deltas_additive():
    n = 120
    x, y = oracle.uniform_instance(n, 77)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 77)
    t2, st = oracle.dvnd(t, D)
    assert st["cost"] == oracle.cost(t2, D) < oracle.cost(t, D)
    # a local optimum: no candidate improves
    for nb in range(5):
        c, _, _, _ = oracle.eval_nb(nb, t2, D)
        assert (c >= 0).all()


def test_legacy_better_no_conflict_quirks():
    moves = [(0, 3, 10, -50), (1, 4, 8, -70), (2, 12, 20, -10), (0, 30, 40, -70), (3, 25, 5, -5)]
    sel, imp, k = oracle.legacy_better_no_conflict(moves)
    assert k == len(sel)
    assert imp == sum(moves[s][3] for s in sel)
    # noConflict(2opt, 2opt) uses (move2.j > move1.i - 1): almost always true
    assert oracle.legacy_no_conflict((1, 5, 9), (1, 6, 8))


def test_solution_checkpoint_text_format(tmp_path, berlin):
    """save_solution / load_solution use the text format of the reference's
    MLSolution::save (tour length, cost, tour on one line)."""
    import mlpgpu

    t = np.array(berlin["random_tour_seed0"], np.int32)
    p = tmp_path / "sol.txt"
    cost = berlin["cost_random_tour_seed0"]
    mlpgpu.save_solution(str(p), t, cost)
    text = p.read_text()
    assert text == f"{len(t)}\n{cost}\n" + " ".join(str(v) for v in t) + "\n"
    t2, c2 = mlpgpu.load_solution(str(p))
    assert np.array_equal(t2, t) and c2 == cost
    (tmp_path / "bad.txt").write_text("53\n1\n0 1 2\n")
    with pytest.raises(ValueError):
        mlpgpu.load_solution(str(tmp_path / "bad.txt"))


@pytest.mark.parametrize("k", [1, 4, 9, 15, 28])
def test_oropt_k_deltas_any_k(k):
    # Or-opt-k of any k in [1, 28] (MLKernelOrOpt(problem, k), move id k + 1):
    # the oracle's per-block candidates match brute force (apply + costCalc).
    n = 70
    x, y = oracle.uniform_instance(n, 30 + k)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 30 + k)
    nb = k + 1
    c, i, j, _ = oracle.eval_nb(nb, t, D)
    assert len(c) == n + 1 - k - 2
    for b in range(len(c)):
        assert c[b] == oracle.move_delta(nb, int(i[b]), int(j[b]), t, D, brute=True)
