"""GPU tests of the sweep timing helper (mlp_solver_time_sweep /
Solver.time_sweep) that bench.py's sweep and roofline figures come from: it
times launches of the solver's own sweep kernel, warm and behind an L2 flush,
and leaves the search where it was."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_time_sweep_times_the_kernel_and_leaves_the_search_unchanged(mlpgpu_mod):
    import torch

    n = 300
    x, y = oracle.uniform_instance(n, 41)
    D = oracle.dist(x, y, True)
    t = oracle.random_perm_tour(n, 41)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    s.set_tour(t)
    warm = s.time_sweep(mlpgpu_mod.NB_ALL, 9)
    flush = torch.empty(64 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")
    cold = s.time_sweep(mlpgpu_mod.NB_ALL, 5, flush.data_ptr(), flush.numel() * 4)
    torch.cuda.synchronize()
    assert 0 < warm < 1e-2 and 0 < cold < 1e-2
    # The tour and the candidate keys are as before: the DVND gives the oracle's optimum.
    assert np.array_equal(s.tour(), t)
    st = s.dvnd()
    ot, ost = oracle.dvnd(t, D)
    assert np.array_equal(s.tour(), ot) and st["cost"] == ost["cost"]


def test_time_sweep_rejects_bad_arguments(mlpgpu_mod):
    x, y = oracle.uniform_instance(20, 3)
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    s.set_tour(oracle.random_perm_tour(20, 3))
    for reps in (0, 5000):
        with pytest.raises(mlpgpu_mod.MLPError):
            s.time_sweep(mlpgpu_mod.NB_ALL, reps)
    with pytest.raises(mlpgpu_mod.MLPError):
        s.time_sweep(mlpgpu_mod.NB_ALL, 3, 12345, 0)
