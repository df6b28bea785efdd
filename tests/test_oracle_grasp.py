"""CPU tests of the oracle's MLSolution::random restatements.

The faithful one (std::sort, as the reference) is pinned by K3 in
test_oracle.py.  The canonical one, which the device constructor follows,
takes equal distances in client-id order; it is checked here against an
independent pure-Python restatement (MTRandom draws from the oracle's pinned
MT19937, rand(max) in IEEE double, ceil(alpha * count) in float32).
"""
import json
import math
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN


def _canonical_py(D, seed, alpha):
    n = D.shape[0]
    raw = iter(oracle.mt_rand(seed, 4 * n + 16).tolist())
    cands = list(range(1, n))
    tour, last = [0], 0
    while cands:
        cnt = len(cands)
        r = 0
        if cnt > 1:
            rcl = int(math.ceil(float(np.float32(alpha) * np.float32(cnt))))
            if rcl > 0:
                r = int(((rcl - 1) + 1.0) * next(raw) / 4294967296.0)
        order = sorted(cands, key=lambda c: (int(D[last, c]), c))
        cur = order[r]
        cands.remove(cur)
        tour.append(cur)
        last = cur
    tour.append(0)
    return np.array(tour, np.int32)


@pytest.mark.parametrize("n,seed,alpha", [(2, 0, 0.5), (3, 1, 0.5), (9, 2, 0.0), (30, 3, 0.3), (52, 0, 0.5),
                                          (120, 4, 1.0), (200, 5, 0.7), (200, 6, 0.1)])
def test_canonical_constructor_matches_python(n, seed, alpha):
    x, y = oracle.clustered_instance(n, 90 + seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_tour_canonical(D, seed, alpha)
    assert t[0] == 0 and t[-1] == 0 and sorted(t[1:-1].tolist()) == list(range(1, n))
    assert np.array_equal(t, _canonical_py(D, seed, alpha))


def test_canonical_equals_faithful_without_ties():
    # alpha = 0.9 on berlin52 (distRound = false): no tie decides a pick.
    berlin = json.load(open(os.path.join(GOLDEN, "berlin52.json")))
    D = oracle.dist(np.array(berlin["x"], np.int32), np.array(berlin["y"], np.int32), False)
    assert np.array_equal(oracle.random_tour_canonical(D, 0, 0.9), oracle.random_tour(D, 0, 0.9))
    # K3's own draw has ties that decide picks: the canonical start differs.
    assert oracle.cost(oracle.random_tour_canonical(D, 0, 0.5), D) != 494309
