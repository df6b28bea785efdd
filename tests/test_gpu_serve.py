"""GPU tests of the serving form (continuous batching, mlp_server_*).

The central property: every served search gives exactly the result it gives
alone (mlp_solver_dvnd on the same instance, start tour, neighbourhood mask and
sweep limit) and, for small instances, the oracle's -- although searches of
different sizes, masks and limits are admitted, iterated and retired in
overlapping groups under a memory budget.  Integer work, so equality is exact.
Failure handling is exercised on the host only: cancellation, rejected
requests and injected admission failures.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

# (n, clustered, neighbourhood mask, sweep limit)
MIX = [
    (40, False, 0x1F, 1 << 20),
    (120, True, 0x1F, 1 << 20),
    (300, False, 0x03, 1 << 20),
    (77, True, 0x1C, 1 << 20),
    (500, True, 0x1F, 40),
    (1900, False, 0x1F, 5),   # merge from the global workspace
    (64, False, 0x1F, 1 << 20),
    (200, True, 0x10, 1 << 20),
    (33, True, 0x01, 1 << 20),
    (640, False, 0x1F, 25),
]


def _instance(q, n, clustered):
    x, y = (oracle.clustered_instance if clustered else oracle.uniform_instance)(n, 300 + q)
    return x, y, oracle.random_perm_tour(n, 300 + q)


def _alone(mlpgpu_mod, x, y, t, mask, limit):
    s = mlpgpu_mod.Solver(mlpgpu_mod.Problem.from_coords(x, y, dist_round=True))
    s.set_tour(t)
    st = s.dvnd(mask, limit)
    return s.tour(), st


def _drain(srv, expect, iters, budget=None, max_active=None):
    out = {}
    for _ in range(100000):
        a, _q = srv.step(iters)
        st = srv.status()
        if budget is not None:
            assert st["mem_in_use"] <= budget
        if max_active is not None:
            assert a <= max_active
        for rid in srv.finished():
            if rid in expect:
                out[rid] = srv.result(rid, expect[rid])
        if len(out) == len(expect):
            return out
    raise AssertionError("server did not drain")


def test_served_results_equal_alone_in_a_staggered_mix(mlpgpu_mod):
    S = mlpgpu_mod.Server
    budget = S.footprint(1900) + S.footprint(640) + S.footprint(120)
    srv = S(budget, wide=False, max_active=3)
    reqs, sizes = {}, {}
    for q, (n, cl, mask, limit) in enumerate(MIX):
        x, y, t = _instance(q, n, cl)
        rid = srv.submit(x, y, t, nb_mask=mask, max_iters=limit)
        reqs[rid] = (x, y, t, mask, limit)
        sizes[rid] = n
    res = _drain(srv, sizes, iters=3, budget=budget, max_active=3)
    assert srv.status()["mem_in_use"] == 0
    for rid, (x, y, t, mask, limit) in reqs.items():
        tour, st, info = res[rid]
        assert info["status"] == 0 and info["n"] == len(x)
        assert info["arrival"] <= info["admitted"] <= info["finished"]
        at, ast = _alone(mlpgpu_mod, x, y, t, mask, limit)
        assert np.array_equal(tour, at), rid
        assert st == ast, (rid, st, ast)
        if len(x) <= 200 and limit == 1 << 20:
            ot, ost = oracle.dvnd(t, oracle.dist(x, y, True), nbs=[nb for nb in range(5) if (mask >> nb) & 1])
            assert np.array_equal(tour, ot) and st["cost"] == ost["cost"], rid


def test_arrivals_join_running_searches(mlpgpu_mod):
    """Requests submitted between steps join searches already on the GPU."""
    srv = mlpgpu_mod.Server(1 << 30, max_active=16)
    first = []
    for q in range(3):
        x, y, t = _instance(50 + q, 400, True)
        first.append((srv.submit(x, y, t), x, y, t))
    srv.step(2)
    late = []
    for q in range(4):
        x, y, t = _instance(60 + q, 90 + 40 * q, False)
        late.append((srv.submit(x, y, t), x, y, t))
    a, _ = srv.step(1)
    assert a >= 5  # both groups active in the same launches
    res = _drain(srv, {rid: len(x) for rid, x, _, _ in first + late}, iters=4)
    for rid, x, y, t in first + late:
        tour, st, _ = res[rid]
        at, ast = _alone(mlpgpu_mod, x, y, t, 0x1F, 1 << 20)
        assert np.array_equal(tour, at) and st == ast


def test_wide_costs_served(mlpgpu_mod):
    srv = mlpgpu_mod.Server(1 << 28, wide=True, max_active=4)
    x, y, t = _instance(7, 150, False)
    rid = srv.submit(x, y, t)
    tour, st, _ = _drain(srv, {rid: 150}, iters=8)[rid]
    ot, ost = oracle.dvnd(t, oracle.dist(x, y, True), wide=True)
    assert np.array_equal(tour, ot) and st["cost"] == ost["cost"]


def test_cancel_injected_failure_and_rejections(mlpgpu_mod):
    S = mlpgpu_mod.Server
    srv = S(S.footprint(300) * 2, max_active=2)
    cases = [_instance(80 + q, 300, q % 2 == 1) for q in range(4)]
    ids = [srv.submit(x, y, t) for x, y, t in cases]
    # Over the whole budget: rejected at submission.
    xb, yb, tb = _instance(90, 1000, False)
    with pytest.raises(mlpgpu_mod.MLPError) as e:
        srv.submit(xb, yb, tb)
    assert e.value.status == 6
    # Malformed tour: rejected at submission.
    bad = cases[0][2].copy()
    bad[3] = bad[4]
    with pytest.raises(mlpgpu_mod.MLPError) as e:
        srv.submit(cases[0][0], cases[0][1], bad)
    assert e.value.status == 1
    srv.cancel(ids[3])                   # still queued: ends at once
    assert srv.result(ids[3], 300)[2]["status"] == mlpgpu_mod.CANCELLED
    srv.step(1)                          # admits ids[0], ids[1]
    assert srv.result(ids[0], 300) is None
    srv.cancel(ids[1])                   # running: retired at the next step
    srv.fail_next_admissions(1)          # ids[2] fails when admitted
    srv.step(1)
    info1 = srv.result(ids[1], 300)[2]
    assert info1["status"] == mlpgpu_mod.CANCELLED
    res = _drain(srv, {ids[0]: 300, ids[2]: 300}, iters=8)
    assert res[ids[2]][2]["status"] == 6
    tour, st, info = res[ids[0]]
    assert info["status"] == 0
    at, ast = _alone(mlpgpu_mod, *cases[0], 0x1F, 1 << 20)
    assert np.array_equal(tour, at) and st == ast
    assert srv.status()["mem_in_use"] == 0
    with pytest.raises(mlpgpu_mod.MLPError):
        srv.result(ids[0], 300)          # already taken
