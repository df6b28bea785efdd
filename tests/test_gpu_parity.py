"""GPU parity tests: every result of the CUDA path is compared bit-for-bit with
the oracle (the CPU restatement of the reference) on the same seeded inputs.

Integer/index work, so the bar is exact equality everywhere (no tolerance).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

BERLIN52 = dict(x=None)


def _berlin():
    import json, os
    from conftest import GOLDEN

    with open(os.path.join(GOLDEN, "berlin52.json")) as f:
        g = json.load(f)
    return np.array(g["x"], np.int32), np.array(g["y"], np.int32), g


@pytest.mark.parametrize("n,seed,rnd", [(5, 1, True), (12, 2, False), (52, 3, True), (200, 4, True), (1000, 5, True)])
def test_dist_matrix(mlpgpu_mod, n, seed, rnd):
    x, y = oracle.uniform_instance(n, seed)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=rnd)
    assert np.array_equal(p.dist(), oracle.dist(x, y, rnd))


@pytest.mark.parametrize("n,seed,wide", [(5, 1, False), (6, 7, False), (7, 2, True), (9, 3, False), (13, 4, False),
                                          (52, 5, False), (101, 6, True), (257, 7, False), (1000, 8, False),
                                          (1000, 9, True)])
def test_candidates_all_neighbourhoods(mlpgpu_mod, n, seed, wide):
    x, y = oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), wide=wide)
    s.set_tour(t)
    assert s.cost() == oracle.cost(t, D, wide)
    assert np.array_equal(s.weights(), oracle.weights(t, D))
    for nb in range(5):
        c, i, j = s.eval(nb)
        oc, oi, oj, _ = oracle.eval_nb(nb, t, D, wide)
        assert np.array_equal(c, oc), f"nb {nb}: deltas differ"
        assert np.array_equal(i, oi) and np.array_equal(j, oj), f"nb {nb}: moves differ"


@pytest.mark.parametrize("shape", range(10))
def test_candidates_every_tile_shape(mlpgpu_mod, shape):
    n = 333
    x, y = oracle.clustered_instance(n, 11)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 11)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    s.set_tile_shape(shape)
    s.set_tour(t)
    for nb in range(5):
        c, i, j = s.eval(nb)
        oc, oi, oj, _ = oracle.eval_nb(nb, t, D)
        assert np.array_equal(c, oc) and np.array_equal(i, oi) and np.array_equal(j, oj)


def test_k4_berlin52_swap_pass(mlpgpu_mod):
    """tests/WamcaExperiment.Test.cpp:70-131: random(rng(0), 0.5) then one swap
    pass (kernel + GPU merge + apply + update) gives 367403."""
    x, y, g = _berlin()
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=False)
    D = oracle.dist(x, y, False)
    t = np.array(g["random_tour_seed0"], np.int32)
    s = mlpgpu_mod.Solver(p)
    s.set_tour(t)
    assert s.cost() == 494309
    new_cost, moves = s.pass_(0)
    assert new_cost == 367403
    ot, oc, omoves = oracle.pass_(0, t, D)
    assert oc == 367403 and moves == omoves and np.array_equal(s.tour(), ot)


@pytest.mark.parametrize("nb", range(5))
def test_pass_each_neighbourhood(mlpgpu_mod, nb):
    n = 300
    x, y = oracle.uniform_instance(n, 20 + nb)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 20 + nb)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    s.set_tour(t)
    new_cost, moves = s.pass_(nb)
    ot, oc, omoves = oracle.pass_(nb, t, D)
    assert new_cost == oc
    assert moves == omoves
    assert np.array_equal(s.tour(), ot)


@pytest.mark.parametrize("n,seed,wide,clustered", [(5, 1, False, False), (8, 2, False, False), (52, 1, False, False),
                                                   (150, 3, True, True), (400, 4, False, True),
                                                   (1000, 5, False, False)])
def test_dvnd_local_optimum(mlpgpu_mod, n, seed, wide, clustered):
    gen = oracle.clustered_instance if clustered else oracle.uniform_instance
    x, y = gen(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), wide=wide)
    s.set_tour(t)
    st = s.dvnd()
    ot, ost = oracle.dvnd(t, D, wide)
    assert np.array_equal(s.tour(), ot)
    assert st["cost"] == ost["cost"] == oracle.cost(ot, D, wide)
    assert st["iterations"] == ost["iterations"]
    assert st["moves"] == ost["moves"]
    assert st["evals"] == ost["evals"]
    assert st["converged"] == 1


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("n,seed,shape", [(5, 11, 0), (6, 12, 2), (7, 13, 8), (9, 14, 3), (13, 15, 1), (37, 16, 9),
                                          (64, 17, 6), (97, 18, 7), (130, 19, 5), (257, 20, 4), (611, 21, 2),
                                          (1000, 22, 3), (5, 23, 10), (8, 24, 11), (11, 25, 12), (66, 26, 13),
                                          (70, 27, 10), (131, 28, 11), (199, 29, 12), (402, 30, 13), (777, 31, 11)])
def test_dvnd_both_sweep_kernels_every_shape(mlpgpu_mod, kernel, n, seed, shape):
    """The DVND through the general fused sweep (0) and through the term-table
    sweep (1) equals the oracle's (tour, cost, iterations, moves, evaluations)
    for tour sizes around every tile edge and each compiled tile shape."""
    x, y = oracle.clustered_instance(n, seed) if n % 2 else oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    s.set_sweep_kernel(kernel)
    s.set_tile_shape(shape)
    s.set_tour(t)
    st = s.dvnd()
    ot, ost = oracle.dvnd(t, D)
    assert np.array_equal(s.tour(), ot)
    assert (st["cost"], st["iterations"], st["moves"], st["evals"]) == \
        (ost["cost"], ost["iterations"], ost["moves"], ost["evals"])


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("n,seed,wide", [(5, 41, False), (9, 42, True), (60, 43, False), (333, 44, True),
                                         (1000, 45, False)])
def test_dvnd_every_merge_kernel(mlpgpu_mod, mode, n, seed, wide):
    """One search's DVND through the six-CTA cluster merge (1) and the one-CTA
    merge (2) equals the oracle's."""
    x, y = oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), wide=wide)
    s.set_merge_mode(mode)
    s.set_tour(t)
    st = s.dvnd()
    ot, ost = oracle.dvnd(t, D, wide)
    assert np.array_equal(s.tour(), ot)
    assert (st["cost"], st["iterations"], st["moves"], st["evals"]) == \
        (ost["cost"], ost["iterations"], ost["moves"], ost["evals"])


def test_dvnd_subset_masks_and_iteration_cap(mlpgpu_mod):
    n = 250
    x, y = oracle.uniform_instance(n, 31)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 31)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    for nbs in ([0], [1], [2, 3, 4], [0, 2], [1, 4]):
        mask = sum(1 << q for q in nbs)
        s.set_tour(t)
        st = s.dvnd(mask)
        ot, ost = oracle.dvnd(t, D, nbs=nbs)
        assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"], nbs
    for cap in (1, 3, 17):
        s.set_tour(t)
        st = s.dvnd(max_iters=cap)
        ot, ost = oracle.dvnd(t, D, max_iters=cap)
        assert st["sweeps"] == cap
        assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"]


def test_ads_buffer_matches_ldsupdate(mlpgpu_mod):
    x, y, g = _berlin()
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=False)
    D = oracle.dist(x, y, False)
    t = np.array(g["random_tour_seed0"], np.int32)
    s = mlpgpu_mod.Solver(p)
    s.set_tour(t)
    a = s.ads()
    o = oracle.ads(t, D, x, y, False)
    assert np.array_equal(a, o)
    ref = np.array(g["ads_random_tour_seed0"], np.uint32)
    assert np.array_equal(a[:6], ref[:6]) and np.array_equal(a[32:], ref[32:])


def test_batch_mixed_sizes_equal_alone(mlpgpu_mod):
    """Each job of a batch gives exactly the result it gives alone (and the oracle's)."""
    sizes = [60, 137, 250, 90, 400, 33]
    b = mlpgpu_mod.Batch()
    cases = []
    for q, n in enumerate(sizes):
        x, y = oracle.clustered_instance(n, 100 + q)
        D = oracle.dist(x, y, True)
        t = oracle.random_perm_tour(n, 100 + q)
        p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
        b.add(p, t)
        cases.append((p, D, t))
    b.run()
    for q, (p, D, t) in enumerate(cases):
        bt, bst = b.result(q)
        ot, ost = oracle.dvnd(t, D)
        assert np.array_equal(bt, ot) and bst["cost"] == ost["cost"], q
        s = mlpgpu_mod.Solver(p)
        s.set_tour(t)
        s.dvnd()
        assert np.array_equal(s.tour(), bt)
    b.reset()
    b.run()
    for q, (p, D, t) in enumerate(cases):
        bt, _ = b.result(q)
        assert np.array_equal(bt, oracle.dvnd(t, D)[0])


def test_matrix_problem_and_errors(mlpgpu_mod):
    n = 40
    x, y = oracle.uniform_instance(n, 41)
    D = oracle.dist(x, y, True)
    p = mlpgpu_mod.Problem.from_matrix(D)
    assert np.array_equal(p.dist(), D)
    s = mlpgpu_mod.Solver(p)
    t = oracle.random_perm_tour(n, 41)
    s.set_tour(t)
    assert np.array_equal(s.tour(), t)
    bad = t.copy()
    bad[3] = bad[4]
    with pytest.raises(mlpgpu_mod.MLPError):
        s.set_tour(bad)
    with pytest.raises(mlpgpu_mod.MLPError):
        s.set_tour(t[:-1])
    Dbad = D.copy()
    Dbad[0, 1] += 1
    with pytest.raises(mlpgpu_mod.MLPError):
        mlpgpu_mod.Problem.from_matrix(Dbad)
    with pytest.raises(mlpgpu_mod.MLPError):
        mlpgpu_mod.Problem.from_coords([0, 1, 2], [0, 1, 2])
    # the solver still works after rejected calls
    s.set_tour(t)
    assert s.dvnd()["cost"] == oracle.dvnd(t, D)[1]["cost"]


@pytest.mark.parametrize("n", [1900, 4200, 4500])
def test_large_sizes_use_global_merge_workspace(mlpgpu_mod, n):
    """The cluster merge's workspace around its shared-memory limit (tour
    size 4419: n = 4418): n = 1900 well inside it; n = 4200 inside it without
    the leader's copy of w (the copy would not fit); n = 4500 beyond it, from a
    global workspace.  Alone and mixed with a small job in one batch."""
    x, y = oracle.uniform_instance(n, 51)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 51)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    s = mlpgpu_mod.Solver(p)
    s.set_tour(t)
    iters = 6 if n < 4000 else 3
    st = s.dvnd(max_iters=iters)
    ot, ost = oracle.dvnd(t, D, max_iters=iters, threads=8)
    assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"]
    b = mlpgpu_mod.Batch()
    xs, ys = oracle.uniform_instance(80, 52)
    Ds = oracle.dist(xs, ys, True)
    ts = oracle.random_perm_tour(80, 52)
    ps = mlpgpu_mod.Problem.from_coords(xs, ys, dist_round=True)
    b.add(ps, ts)
    b.add(p, t)
    b.run(max_iters=iters)
    assert np.array_equal(b.result(0)[0], oracle.dvnd(ts, Ds, max_iters=iters)[0])
    assert np.array_equal(b.result(1)[0], ot)


def test_large_n10000_wide_candidates_and_capped_dvnd(mlpgpu_mod):
    """n = 10000 with int64 costs (400 MB distance matrix in HBM): cost,
    2-opt and Or-opt-3 candidates and a DVND capped at two sweeps, all equal
    to the oracle's."""
    import os

    n = 10000
    x, y = oracle.uniform_instance(n, 2025)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 5)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), wide=True)
    s.set_tour(t)
    assert s.cost() == oracle.cost(t, D, True)
    for nb in (1, 4):
        c, i, j = s.eval(nb)
        oc, oi, oj, _ = oracle.eval_nb(nb, t, D, True)
        assert np.array_equal(c, oc) and np.array_equal(i, oi) and np.array_equal(j, oj), nb
    st = s.dvnd(mlpgpu_mod.NB_ALL, 2)
    ot, ost = oracle.dvnd(t, D, wide=True, max_iters=2, threads=os.cpu_count() or 1)
    assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"] and st["moves"] == ost["moves"]


def test_batch_merge_kernels_give_identical_results(mlpgpu_mod):
    """The one-CTA-per-job merge (large batches) and the six-CTA cluster merge
    select and apply the same moves: 20 jobs of mixed sizes, including one
    whose one-CTA merge runs from a global workspace (n = 3200), agree with
    each other, with the plain solver and with the oracle."""
    sizes = [30, 45, 60, 77, 90, 101, 120, 150, 180, 200, 230, 260, 300, 350, 400, 480, 560, 700, 1200, 3200]
    cases = []
    for q, n in enumerate(sizes):
        x, y = (oracle.clustered_instance if q % 2 else oracle.uniform_instance)(n, 900 + q)
        cases.append((mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), x, y, oracle.random_perm_tour(n, 900 + q)))
    limit = 12
    out = {}
    for mode in (1, 2, 0):
        b = mlpgpu_mod.Batch()
        b.set_merge_mode(mode)
        for p, _, _, t in cases:
            b.add(p, t)
        b.run(max_iters=limit)
        out[mode] = [b.result(j) for j in range(len(cases))]
    for j in range(len(cases)):
        (t1, s1), (t2, s2), (t0, s0) = out[1][j], out[2][j], out[0][j]
        assert np.array_equal(t1, t2) and s1 == s2, j
        assert np.array_equal(t0, t1) and s0 == s1, j
    for j in (0, 5, 11, 19):
        p, x, y, t = cases[j]
        s = mlpgpu_mod.Solver(p)
        s.set_tour(t)
        st = s.dvnd(max_iters=limit)
        assert np.array_equal(s.tour(), out[2][j][0]) and st == out[2][j][1], j
    for j in (0, 3, 9):
        p, x, y, t = cases[j]
        ot, ost = oracle.dvnd(t, oracle.dist(x, y, True), max_iters=limit)
        assert np.array_equal(out[2][j][0], ot) and out[2][j][1]["cost"] == ost["cost"], j


@pytest.mark.parametrize("wide", [False, True])
def test_batch_tiny_and_mixed_sizes_with_int64_costs(mlpgpu_mod, wide):
    """Edge sizes in the batched path: the smallest tours (n = 5 .. 12) next to
    larger ones, 32-bit and 64-bit costs, the one-CTA merge (20 jobs) --
    every job equal to the oracle's DVND."""
    sizes = [5, 6, 7, 8, 9, 10, 11, 12, 13, 17, 23, 31, 40, 55, 64, 90, 128, 150, 201, 260]
    b = mlpgpu_mod.Batch(wide=wide)
    cases = []
    for q, n in enumerate(sizes):
        x, y = oracle.uniform_instance(n, 1300 + q)
        t = oracle.random_perm_tour(n, 1300 + q)
        b.add(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), t)
        cases.append((oracle.dist(x, y, True), t))
    b.run()
    for j, (D, t) in enumerate(cases):
        bt, bst = b.result(j)
        ot, ost = oracle.dvnd(t, D, wide=wide)
        assert np.array_equal(bt, ot) and bst["cost"] == ost["cost"] and bst["moves"] == ost["moves"], sizes[j]


def test_checkpoint_resume_continues_the_same_search(mlpgpu_mod, tmp_path):
    """A DVND stopped after some sweeps, saved in MLSolution's text format and
    resumed in a new solver ends where the uninterrupted search ends."""
    n = 400
    x, y = oracle.uniform_instance(n, 88)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    t = oracle.random_perm_tour(n, 88)
    full = mlpgpu_mod.Solver(p)
    full.set_tour(t)
    st_full = full.dvnd()
    a = mlpgpu_mod.Solver(p)
    a.set_tour(t)
    st_a = a.dvnd(max_iters=20)
    path = str(tmp_path / "ck.txt")
    a.save(path)
    tour_saved, cost_saved = mlpgpu_mod.load_solution(path)
    assert np.array_equal(tour_saved, a.tour()) and cost_saved == st_a["cost"]
    b = mlpgpu_mod.Solver(p)
    b.load(path)
    assert b.cost() == st_a["cost"]
    st_b = b.dvnd()
    assert np.array_equal(b.tour(), full.tour()) and st_b["cost"] == st_full["cost"]
    assert st_a["sweeps"] + st_b["sweeps"] == st_full["sweeps"]
    # A length written without the trailing depot (size - 1) is accepted, as
    # the reference's loader does; the tour read is still size entries long.
    bad = tmp_path / "short.txt"
    bad.write_text(f"{n}\n0\n" + " ".join(str(v) for v in t) + "\n")
    c = mlpgpu_mod.Solver(p)
    c.load(str(bad))
    assert np.array_equal(c.tour(), t)
    (tmp_path / "trunc.txt").write_text(f"{n + 1}\n0\n0 1 2\n")
    with pytest.raises(mlpgpu_mod.MLPError):
        c.load(str(tmp_path / "trunc.txt"))
