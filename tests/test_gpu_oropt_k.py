"""GPU parity tests of Or-opt-k for any k in [1, 28] (MLKernelOrOpt(problem,
k), move id k + 1): per-block candidates and one pass (greedy merge with
f_canOrOptMerge, apply, update) against the oracle, bit-exact."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _solver(mlpgpu_mod, n, seed, wide):
    x, y = oracle.uniform_instance(n, seed)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, seed)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True), wide=wide)
    s.set_tour(t)
    return s, t, D


@pytest.mark.parametrize("n,wide", [(40, False), (300, False), (300, True), (1000, False)])
@pytest.mark.parametrize("k", [1, 2, 3, 4, 7, 15, 28])
def test_oropt_k_candidates(mlpgpu_mod, n, wide, k):
    s, t, D = _solver(mlpgpu_mod, n, 50 + k, wide)
    c, i, j = s.eval_oropt(k)
    oc, oi, oj, _ = oracle.eval_nb(k + 1, t, D, wide)
    assert np.array_equal(c, oc) and np.array_equal(i, oi) and np.array_equal(j, oj)
    if k <= 3:  # the fused sweep's Or-opt-k slot gives the same candidates
        fc, fi, fj = s.eval(k + 1)
        assert np.array_equal(fc, c) and np.array_equal(fi, i) and np.array_equal(fj, j)


@pytest.mark.parametrize("n,wide", [(60, False), (500, True), (1000, False)])
@pytest.mark.parametrize("k", [1, 3, 5, 12, 28])
def test_oropt_k_pass(mlpgpu_mod, n, wide, k):
    s, t, D = _solver(mlpgpu_mod, n, 80 + k, wide)
    new_cost, moves = s.pass_oropt(k)
    ot, oc, omoves = oracle.pass_(k + 1, t, D, wide)
    assert moves == omoves
    assert new_cost == oc
    assert np.array_equal(s.tour(), ot)
    # the solver continues from the new tour (ADS rebuilt)
    st = s.dvnd(0x1F, 3)
    ot2, ost2 = oracle.dvnd(ot, D, wide, max_iters=3)
    assert np.array_equal(s.tour(), ot2) and st["cost"] == ost2["cost"]


def test_oropt_k_rejects_bad_k(mlpgpu_mod):
    s, _, _ = _solver(mlpgpu_mod, 20, 1, False)
    for k in (0, 29, 19):
        with pytest.raises(mlpgpu_mod.MLPError):
            s.eval_oropt(k)
