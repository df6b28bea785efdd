"""GPU test of mlp_eval_noalloc, the evaluation entry point that allocates no
device memory (for callers that cannot call cudaMalloc: code inside another
framework's memory pool or budget, or hosts that must not synchronise the
device with allocations).  Its candidates must equal the oracle's and those of
the existing entry point (mlp_solver_eval) exactly, call after call, although
every call reuses the library's one fixed scratch array.  Sizes cover the
smallest tour (n = 5), a middle one and the largest the array holds
(n = 2047, where its layout is tightest), in both cost widths.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _count(nb: int, n: int) -> int:
    """Candidate count of neighbourhood nb (the formula the header states)."""
    size = n + 1
    if nb == 0:
        return (size + 1) // 2 - 1
    if nb == 1:
        return (size + 1) // 2
    return size - (nb - 1) - 2


def _call(mlpgpu_mod, torch, D, n, tour, nb, wide):
    m = _count(nb, n)
    t_dev = _dev(torch, tour)
    cost = torch.empty(m, dtype=torch.int64, device="cuda")
    ci = torch.empty(m, dtype=torch.int32, device="cuda")
    cj = torch.empty(m, dtype=torch.int32, device="cuda")
    mlpgpu_mod.eval_noalloc(D.data_ptr(), n, t_dev.data_ptr(), nb, wide, cost.data_ptr(), ci.data_ptr(),
                            cj.data_ptr(), 0)
    torch.cuda.synchronize()
    return cost.cpu().numpy(), ci.cpu().numpy(), cj.cpu().numpy()


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("n", [5, 300, 2047])
def test_noalloc_matches_oracle_and_solver_eval_on_consecutive_calls(mlpgpu_mod, n, wide):
    torch = pytest.importorskip("torch")
    x, y = oracle.uniform_instance(n, 61)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    Dh = p.dist()
    s = mlpgpu_mod.Solver(p, wide=wide)
    D = _dev(torch, Dh)
    tours = [oracle.random_perm_tour(n, 61), oracle.random_perm_tour(n, 62)]
    calls = [(0, 1), (1, 4), (1, 4), (0, 0), (1, 2), (0, 3)]  # (tour index, neighbourhood), back to back
    for ti, nb in calls:
        assert s.num_candidates(nb) == _count(nb, n)
        c, i, j = _call(mlpgpu_mod, torch, D, n, tours[ti], nb, wide)
        oc, oi, oj, _ = oracle.eval_nb(nb, tours[ti], Dh, wide=wide)
        assert np.array_equal(c, oc), (ti, nb)
        assert np.array_equal(i, oi) and np.array_equal(j, oj), (ti, nb)
        s.set_tour(tours[ti])
        ec, ei, ej = s.eval(nb)
        assert np.array_equal(c, ec) and np.array_equal(i, ei) and np.array_equal(j, ej), (ti, nb)


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


@pytest.mark.parametrize("bad", ["client_out_of_range", "negative", "repeated_client", "depot_moved"])
def test_noalloc_flags_malformed_tours_before_reading_distances(mlpgpu_mod, bad):
    """A malformed tour is caught by the device-side check before any distance
    is gathered through it (no out-of-range access), every output entry
    becomes (INT64_MIN, -1, -1), and the next call with a good tour is exact."""
    torch = pytest.importorskip("torch")
    n = 64
    x, y = oracle.uniform_instance(n, 5)
    p = mlpgpu_mod.Problem.from_coords(x, y, dist_round=True)
    Dh = p.dist()
    D = _dev(torch, Dh)
    good = oracle.random_perm_tour(n, 5)
    t = good.copy()
    if bad == "client_out_of_range":
        t[7] = n + 1000
    elif bad == "negative":
        t[3] = -5
    elif bad == "repeated_client":
        t[9] = t[10]
    else:
        t[0], t[4] = t[4], t[0]
    for nb in (0, 2):
        c, i, j = _call(mlpgpu_mod, torch, D, n, t, nb, False)
        assert (c == np.iinfo(np.int64).min).all() and (i == -1).all() and (j == -1).all()
    c, i, j = _call(mlpgpu_mod, torch, D, n, good, 1, False)
    oc, oi, oj, _ = oracle.eval_nb(1, good, Dh, wide=False)
    assert np.array_equal(c, oc) and np.array_equal(i, oi) and np.array_equal(j, oj)
