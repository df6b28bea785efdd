"""GPU parity tests of the device multi-start constructor (MLSolution::random
with equal distances in client-id order): Problem.random_tours,
Solver.random_tour and Batch.add_random against the oracle's canonical
restatement, bit-exact."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,clustered", [(5, False), (6, True), (9, False), (52, True), (300, False), (1000, True),
                                         (2500, False)])
@pytest.mark.parametrize("alpha", [0.0, 0.1, 0.5, 0.9, 1.0])
def test_random_tours_match_oracle(mlpgpu_mod, n, clustered, alpha):
    x, y = (oracle.clustered_instance if clustered else oracle.uniform_instance)(n, 11)
    D = oracle.dist(x, y, True)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    seeds = [0, 1, 7, 123456789, 4294967295]
    tours = p.random_tours(seeds, alpha)
    for q, sd in enumerate(seeds):
        assert np.array_equal(tours[q], oracle.random_tour_canonical(D, sd, alpha)), (sd, alpha)


def test_berlin52_and_many_starts(mlpgpu_mod):
    x, y = oracle.uniform_instance(400, 3)
    D = oracle.dist(x, y, False)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=False)
    seeds = list(range(100, 180))
    tours = p.random_tours(seeds, 0.5)
    for q, sd in enumerate(seeds):
        assert np.array_equal(tours[q], oracle.random_tour_canonical(D, sd, 0.5))


def test_solver_and_batch_start_on_the_device(mlpgpu_mod):
    x, y = oracle.clustered_instance(350, 5)
    D = oracle.dist(x, y, True)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    s = mlpgpu_mod.Solver(p)
    s.random_tour(42, 0.5)
    t0 = oracle.random_tour_canonical(D, 42, 0.5)
    assert np.array_equal(s.tour(), t0) and s.cost() == oracle.cost(t0, D)
    st = s.dvnd()
    ot, ost = oracle.dvnd(t0, D)
    assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"]
    b = mlpgpu_mod.Batch()
    for sd in (1, 2, 3, 4):
        b.add_random(p, sd, 0.3)
    b.run()
    for q, sd in enumerate((1, 2, 3, 4)):
        bt, bst = b.result(q)
        ot, ost = oracle.dvnd(oracle.random_tour_canonical(D, sd, 0.3), D)
        assert np.array_equal(bt, ot) and bst["cost"] == ost["cost"], sd
    with pytest.raises(mlpgpu_mod.MLPError):
        s.random_tour(1, 1.5)
