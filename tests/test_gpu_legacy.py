"""GPU tests of the reference's legacy extern "C" DVND entry points
(include/wamca_dvnd.h): bestNeighbor / bestNeighborSimple / applyMoves with
the reference's semantics, against the oracle, bit-exact.  Instances are
TSPLIB files loaded with costTour = true, distRound = false (dvnd.cpp:163-175)."""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _tsp(path, x, y, name):
    lines = [f"NAME : {name}", "TYPE : TSP", f"DIMENSION : {len(x)}", "EDGE_WEIGHT_TYPE : EUC_2D",
             "NODE_COORD_SECTION"] + [f"{q + 1} {a} {b}" for q, (a, b) in enumerate(zip(x, y))] + ["EOF"]
    path.write_text("\n".join(lines) + "\n")
    return str(path)


def _berlin(tmp_path):
    b = json.load(open(os.path.join(GOLDEN, "berlin52.json")))
    x, y = np.array(b["x"], np.int32), np.array(b["y"], np.int32)
    return _tsp(tmp_path / "berlin52.tsp", x, y, "berlin52"), oracle.dist(x, y, False)


@pytest.fixture(autouse=True)
def _fresh(mlpgpu_mod):
    mlpgpu_mod.Legacy.reset()  # the reference caches its first file for the process
    yield
    mlpgpu_mod.Legacy.reset()


def test_best_neighbor_known_answers_and_every_neighbourhood(mlpgpu_mod, tmp_path):
    L = mlpgpu_mod.Legacy
    path, D = _berlin(tmp_path)
    t = oracle.random_tour(D, 0, 0.5)  # K3 start
    r, _ = L.best_neighbor(path, t.copy(), 0, just_calc=True)
    assert r == 494309  # K3
    sol = t.astype(np.int32).copy()
    r, _ = L.best_neighbor(path, sol, 0)
    assert r == 367403  # K4: one swap pass, the tour overwritten in place
    ot, oc, _ = oracle.pass_(0, t, D)
    assert np.array_equal(sol, ot)
    for nb in range(5):
        sol = t.astype(np.int32).copy()
        resp = np.zeros_like(sol)
        r, moves = L.best_neighbor(path, sol, nb, use_moves=1000, solution_resp=resp)
        ot, oc, om = oracle.pass_(nb, t, D)
        assert r == oc and np.array_equal(resp, ot), nb
        assert np.array_equal(sol, t), nb  # left unchanged when moves are requested
        assert moves == [(i_d, i, j, c) for i_d, i, j, c in om], nb
    # a cap below the number applied truncates the vectors
    r, moves = L.best_neighbor(path, t.astype(np.int32).copy(), 0, use_moves=2,
                               solution_resp=np.zeros(len(t), np.int32))
    assert len(moves) == 2 and r == 367403


def test_best_neighbor_keeps_its_first_file(mlpgpu_mod, tmp_path):
    L = mlpgpu_mod.Legacy
    path_a, Da = _berlin(tmp_path)
    x, y = oracle.uniform_instance(52, 4)
    path_b = _tsp(tmp_path / "other.tsp", x, y, "other")
    Db = oracle.dist(x, y, False)
    t = oracle.random_perm_tour(52, 4)
    L.best_neighbor(path_a, t.copy(), 0, just_calc=True)
    r, _ = L.best_neighbor(path_b, t.copy(), 0, just_calc=True)
    assert r == oracle.cost(t, Da)  # dvnd.cu:23: the first file, for the life of the process
    L.reset()
    r, _ = L.best_neighbor(path_b, t.copy(), 0, just_calc=True)
    assert r == oracle.cost(t, Db)


def test_best_neighbor_simple_and_apply_moves(mlpgpu_mod, tmp_path):
    L = mlpgpu_mod.Legacy
    path, D = _berlin(tmp_path)
    t = oracle.random_tour(D, 0, 0.5)
    sol = t.astype(np.int32).copy()
    r = mlpgpu_mod.lib().bestNeighborSimple(path.encode(), mlpgpu_mod._ptr(sol), len(sol), 2)
    ot, oc, _ = oracle.pass_(2, t, D)
    assert r == oc and np.array_equal(sol, ot)
    # applyMoves: moves in order, 2-opt ids applied as swaps (dvnd.cpp:51-75)
    moves = []
    for nb in range(5):
        moves += [(i_d, i, j, c) for i_d, i, j, c in oracle.pass_(nb, t, D)[2][:2]]
    sol = t.astype(np.int32).copy()
    r = L.apply_moves(path, sol, moves)
    et, ec = oracle.legacy_apply_moves(t, D, moves)
    assert np.array_equal(sol, et) and r == ec
