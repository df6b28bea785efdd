"""GPU test of mlp_eval_noalloc, the evaluation entry point that allocates no
device memory (for callers that cannot call cudaMalloc: code inside another
framework's memory pool or budget, or hosts that must not synchronise the
device with allocations).  Its candidates must equal those of the existing
entry point (mlp_solver_eval) exactly, call after call, although every call
reuses the library's one fixed scratch array.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("wide", [False, True])
def test_noalloc_matches_solver_eval_on_consecutive_calls(mlpgpu_mod, wide):
    torch = pytest.importorskip("torch")
    n = 300
    x, y = oracle.uniform_instance(n, 61)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    s = mlpgpu_mod.Solver(p, wide=wide)
    D = _dev(torch, p.dist())
    tours = [oracle.random_perm_tour(n, 61), oracle.random_perm_tour(n, 62)]
    calls = [(0, 1), (1, 4), (1, 4), (0, 0), (1, 2), (0, 3)]  # (tour index, neighbourhood), back to back
    for ti, nb in calls:
        m = s.num_candidates(nb)
        t_dev = _dev(torch, tours[ti])
        cost = torch.empty(m, dtype=torch.int64, device="cuda")
        ci = torch.empty(m, dtype=torch.int32, device="cuda")
        cj = torch.empty(m, dtype=torch.int32, device="cuda")
        mlpgpu_mod.eval_noalloc(D.data_ptr(), n, t_dev.data_ptr(), nb, wide, cost.data_ptr(), ci.data_ptr(),
                                cj.data_ptr(), 0)
        torch.cuda.synchronize()
        s.set_tour(tours[ti])
        ec, ei, ej = s.eval(nb)
        assert np.array_equal(cost.cpu().numpy(), ec), (ti, nb)
        assert np.array_equal(ci.cpu().numpy(), ei) and np.array_equal(cj.cpu().numpy(), ej), (ti, nb)


def test_noalloc_rejects_instances_beyond_its_capacity(mlpgpu_mod):
    torch = pytest.importorskip("torch")
    n = 2100
    D = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    t = _dev(torch, oracle.random_perm_tour(n, 1))
    out = torch.empty(4 * n, dtype=torch.int64, device="cuda")
    with pytest.raises(mlpgpu_mod.MLPError) as e:
        mlpgpu_mod.eval_noalloc(D.data_ptr(), n, t.data_ptr(), 0, False, out.data_ptr(), out.data_ptr(),
                                out.data_ptr(), 0)
    assert e.value.status == 3
