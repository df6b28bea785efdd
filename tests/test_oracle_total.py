"""CPU tests of the oracle's TOTAL multi-improvement (every evaluated move is
a merge candidate; MLKernel isTotal, mlkernel.cu:183-250).

The oracle's TOTAL greedy is checked against an independent pure-Python
restatement on small tours: every distinct move of the ODC kernels' mapping,
its delta by brute force (apply the move, recompute the latency), the sort on
(delta, i, j), the greedy with the same-neighbourhood predicate.  Properties
at larger sizes: the kept set is independent, the latency changes by the sum
of the kept deltas, and the TOTAL DVND ends in a local optimum of every
neighbourhood.
"""
import numpy as np
import pytest

import oracle


def _odc_move(nb, size, by, ctx):
    """(block, thread) -> (i, j) of the ODC kernels with costTour = 1
    (mlkswap.cu:766-768, mlk2opt.cu:561-563, mlkoropt.cu:701-722)."""
    k = ctx >= by
    if nb == 0:
        return (by + 1, ctx + 3) if k else (size - by - 3, size - ctx - 2)
    if nb == 1:
        return (ctx - by + 1, ctx + 2) if k else (by - ctx, size - ctx - 2)
    kk = nb - 1
    return (ctx - by + 1, ctx + 2) if k else (size - ctx - kk - 1, by - ctx)


def _brute_total(nb, tour, D, wide):
    size = len(tour)
    seen, cands = set(), []
    for by in range(oracle.num_blocks(nb, size)):
        for ctx in range(oracle.num_threads(nb, size)):
            i, j = _odc_move(nb, size, by, ctx)
            if (i, j) in seen:
                continue
            seen.add((i, j))
            d = oracle.move_delta(nb, i, j, tour, D, wide=wide, brute=True)
            if d < 0:
                cands.append((d, i, j))
    cands.sort()
    kept = []
    for d, i, j in cands:
        if all(oracle.can_merge_same(nb, (nb, ki, kj), (nb, i, j)) for _, ki, kj in kept):
            kept.append((d, i, j))
    return kept, len(cands)


@pytest.mark.parametrize("n,seed,wide", [(6, 1, False), (9, 2, False), (14, 3, True), (23, 4, False), (31, 5, False)])
def test_total_greedy_matches_brute_force(n, seed, wide):
    x, y = oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    for nb in range(5):
        kept, nc = oracle.total_select(nb, t, D, wide)
        bkept, bnc = _brute_total(nb, t, D, wide)
        assert nc == bnc, nb
        assert kept == bkept, nb


@pytest.mark.parametrize("nb", range(5))
def test_total_pass_is_independent_and_additive(nb):
    n = 400
    x, y = oracle.clustered_instance(n, 40 + nb)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 40 + nb)
    kept, nc = oracle.total_select(nb, t, D)
    assert 0 < len(kept) <= nc
    for a in range(len(kept)):
        for b in range(a):
            assert oracle.can_merge_same(nb, (nb, kept[b][1], kept[b][2]), (nb, kept[a][1], kept[a][2]))
    nt, nc2, moves = oracle.total_pass(nb, t, D)
    assert [(c, i, j) for _, i, j, c in moves] == kept
    assert nc2 == oracle.cost(t, D) + sum(c for c, _, _ in kept)
    assert nc2 == oracle.cost(nt, D)


def test_total_dvnd_reaches_a_local_optimum():
    n = 120
    x, y = oracle.uniform_instance(n, 9)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 9)
    tt, st = oracle.dvnd_total(t, D)
    assert st["cost"] == oracle.cost(tt, D) < oracle.cost(t, D)
    assert st["evals"] == (st["iterations"] + 1) * oracle.evals_per_sweep(n + 1)
    for nb in range(5):
        kept, nc = oracle.total_select(nb, tt, D)
        assert nc == 0 and kept == []
    t2, st2 = oracle.dvnd(tt, D)
    assert np.array_equal(t2, tt) and st2["moves"] == 0
