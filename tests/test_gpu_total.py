"""GPU parity tests of the TOTAL multi-improvement (Solver.set_total /
Batch.set_total): every move a neighbourhood evaluates is a merge candidate.

The collecting sweep, the batched TOTAL greedy (mlp_total.cu) and the
cross-neighbourhood finish must give exactly the oracle's kept moves, tours
and latencies -- integer work, so equality is exact, in 32-bit wrap-around
and 64-bit cost modes.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _setup(mlpgpu_mod, n, seed, clustered=False, wide=False):
    gen = oracle.clustered_instance if clustered else oracle.uniform_instance
    x, y = gen(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), wide=wide)
    s.set_total(True)
    s.set_tour(t)
    return s, t, D


@pytest.mark.parametrize("n,seed,wide", [(5, 1, False), (8, 2, True), (40, 3, False), (300, 4, False),
                                         (300, 5, True), (1000, 6, False)])
@pytest.mark.parametrize("nb", range(5))
def test_total_pass_each_neighbourhood(mlpgpu_mod, n, seed, wide, nb):
    s, t, D = _setup(mlpgpu_mod, n, seed + 10 * nb, wide=wide)
    new_cost, moves = s.pass_(nb)
    ot, oc, omoves = oracle.total_pass(nb, t, D, wide)
    assert moves == omoves
    assert new_cost == oc
    assert np.array_equal(s.tour(), ot)


@pytest.mark.parametrize("n,seed,wide,clustered,mask", [(6, 1, False, False, 0x1F), (52, 2, False, True, 0x1F),
                                                        (150, 3, True, False, 0x1F), (250, 4, False, True, 0x1F),
                                                        (200, 5, False, False, 0x06), (180, 6, True, True, 0x19)])
def test_total_dvnd_matches_oracle(mlpgpu_mod, n, seed, wide, clustered, mask):
    s, t, D = _setup(mlpgpu_mod, n, seed, clustered, wide)
    st = s.dvnd(mask)
    nbs = [nb for nb in range(5) if (mask >> nb) & 1]
    ot, ost = oracle.dvnd_total(t, D, wide, nbs=nbs)
    assert np.array_equal(s.tour(), ot)
    assert st["cost"] == ost["cost"]
    assert st["converged"] == 1
    assert st["moves"] == ost["moves"]
    assert st["sweeps"] == ost["iterations"] + 1
    assert st["evals"] == ost["evals"]


def test_total_dvnd_n1000_capped_and_mode_switch(mlpgpu_mod):
    s, t, D = _setup(mlpgpu_mod, 1000, 21)
    st = s.dvnd(0x1F, 12)
    ot, ost = oracle.dvnd_total(t, D, max_iters=12)
    assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"]
    # Back to per-block candidates: the canonical DVND continues from here.
    s.set_total(False)
    st2 = s.dvnd(0x1F, 10)
    ot2, ost2 = oracle.dvnd(ot, D, max_iters=10)
    assert np.array_equal(s.tour(), ot2) and st2["cost"] == ost2["cost"]


def test_total_batch_equals_alone(mlpgpu_mod):
    b = mlpgpu_mod.Batch()
    b.set_total(True)
    cases = []
    for q, n in enumerate([30, 77, 140, 260, 33, 190]):
        x, y = (oracle.clustered_instance if q % 2 else oracle.uniform_instance)(n, 70 + q)
        t = oracle.random_perm_tour(n, 70 + q)
        b.add(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), t)
        cases.append((x, y, t))
    b.run()
    for q, (x, y, t) in enumerate(cases):
        ot, ost = oracle.dvnd_total(t, oracle.dist(x, y, True))
        bt, bst = b.result(q)
        assert np.array_equal(bt, ot), q
        assert bst["cost"] == ost["cost"] and bst["moves"] == ost["moves"], q


@pytest.mark.parametrize("count,wide", [(20, False), (70, True)])
def test_total_batch_cluster_widths(mlpgpu_mod, count, wide):
    # The greedy streams each list with a cluster of 8 CTAs for a few jobs and
    # narrows the clusters as the batch grows (2 CTAs at 20 jobs, 1 at 70):
    # every width gives the oracle's tours.
    b = mlpgpu_mod.Batch(wide=wide)
    b.set_total(True)
    cases = []
    for q in range(count):
        n = 12 + (q * 37) % 90
        x, y = (oracle.clustered_instance if q % 3 == 0 else oracle.uniform_instance)(n, 300 + q)
        t = oracle.random_perm_tour(n, 300 + q)
        b.add(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), t)
        cases.append((x, y, t))
    b.run()
    for q, (x, y, t) in enumerate(cases):
        ot, ost = oracle.dvnd_total(t, oracle.dist(x, y, True), wide)
        bt, bst = b.result(q)
        assert np.array_equal(bt, ot), q
        assert bst["cost"] == ost["cost"] and bst["moves"] == ost["moves"], q


@pytest.mark.parametrize("wide,nbs,iters", [(False, [0, 1], 2), (True, [1, 4], 1)])
def test_total_large_size_global_workspace(mlpgpu_mod, wide, nbs, iters):
    # n = 2500: the finish runs from the job's global merge workspace (the
    # stage-3 list no longer fits shared memory), the lists hold millions of keys.
    s, t, D = _setup(mlpgpu_mod, 2500, 9, wide=wide)
    mask = sum(1 << nb for nb in nbs)
    st = s.dvnd(mask, iters)
    ot, ost = oracle.dvnd_total(t, D, wide, nbs=nbs, max_iters=iters)
    assert np.array_equal(s.tour(), ot)
    assert st["cost"] == ost["cost"] and st["moves"] == ost["moves"]


def test_total_dvnd_device_loop_and_async(mlpgpu_mod):
    # The three TOTAL kernels captured in the CUDA graph's conditional while
    # node (set_unroll(0)) and the enqueued form give the host loop's result.
    s, t, D = _setup(mlpgpu_mod, 180, 12)
    ot, ost = oracle.dvnd_total(t, D)
    s.set_unroll(0)
    st = s.dvnd()
    assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"] and st["converged"] == 1
    s.set_tour(t)
    s.dvnd_async()
    st2 = s.stats()
    assert np.array_equal(s.tour(), ot) and st2["cost"] == ost["cost"]
