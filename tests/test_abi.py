"""CPU tests of the C-ABI library: it loads, and it exports every function the
public headers declare (no compute calls: there is no GPU here)."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(ROOT, "wamca-gpu-mi_gb300", "lib", "libmlpgpu.so")


def declared_functions():
    names = set()
    for h in os.listdir(INCLUDE):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(INCLUDE, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"MLP_API\s+[\w\s\*]+?\b(\w+)\s*\(", src):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def built_lib():
    if not os.path.exists(LIB):
        import build_lib

        build_lib.build()
    return LIB


def test_headers_declare_the_reference_boundary():
    names = declared_functions()
    for legacy in ("bestNeighborSimple", "bestNeighbor", "applyMoves", "getNoConflictMoves", "noConflict",
                   "segFault"):
        assert legacy in names
    assert "mlp_solver_dvnd" in names and "mlp_batch_run" in names


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = declared_functions() - exported
    assert not missing, missing


def test_library_loads_and_reports_status(built_lib):
    import mlpgpu

    L = mlpgpu.lib()
    assert L.mlp_version() >= 10000
    assert L.mlp_status_string(0) == b"ok"
    assert L.mlp_status_string(3) == b"value out of range"


def test_host_side_legacy_predicates_match_oracle(built_lib):
    """noConflict / getNoConflictMoves are host-side in the reference too."""
    import mlpgpu
    import oracle
    import numpy as np

    rng = np.random.default_rng(5)
    for _ in range(3000):
        a = (int(rng.integers(0, 5)), int(rng.integers(1, 40)), int(rng.integers(1, 40)))
        b = (int(rng.integers(0, 5)), int(rng.integers(1, 40)), int(rng.integers(1, 40)))
        assert mlpgpu.Legacy.no_conflict(*a, *b) == oracle.legacy_no_conflict(a, b)
    for trial in range(200):
        m = int(rng.integers(0, 30))
        moves = [(int(rng.integers(0, 5)), int(rng.integers(1, 60)), int(rng.integers(1, 60)),
                  int(rng.integers(-100, 20))) for _ in range(m)]
        for mx in (False, True):
            for mpp in (False, True):
                got = mlpgpu.Legacy.no_conflict_moves(moves, mx, mpp)
                exp = oracle.legacy_better_no_conflict(moves, mx, mpp)
                assert got == exp


def test_segfault_raises_sigsegv_in_a_child_process(built_lib):
    code = ("import sys; sys.path.insert(0, %r); import mlpgpu; mlpgpu.lib().segFault()"
            % os.path.join(ROOT, "wamca-gpu-mi_gb300"))
    r = subprocess.run(["python3", "-c", code], capture_output=True)
    assert r.returncode == -11


def test_tuning_table_set_get_load_and_validation(tmp_path):
    """The autotuner's tile-shape table: round trip, JSON loading (the format
    mlpgpu/autotune.py writes) and rejection of malformed tables.  Host-only
    calls (no GPU work)."""
    import json

    mlpgpu = pytest.importorskip("mlpgpu")
    saved = mlpgpu.tuning_table()
    try:
        mlpgpu.set_tuning_table([(101, 0, 4), (1001, 3, 4), (16384, 7, 7)])
        assert mlpgpu.tuning_table() == [(101, 0, 4), (1001, 3, 4), (16384, 7, 7)]
        p = tmp_path / "t.json"
        p.write_text(json.dumps({"device": "x", "table": [[201, 1, 2], [5001, 3, 7]],
                                 "timings": [{"n": 200, "one_s": {"0": 0.1}}]}, indent=1))
        assert mlpgpu.lib().mlp_tuning_load(str(p).encode()) == 0
        assert mlpgpu.tuning_table() == [(201, 1, 2), (5001, 3, 7)]
        for bad in ([(101, 0, 14)], [(1001, 0, 1), (101, 0, 1)], [(0, 0, 0)]):
            with pytest.raises(mlpgpu.MLPError):
                mlpgpu.set_tuning_table(bad)
        assert mlpgpu.tuning_table() == [(201, 1, 2), (5001, 3, 7)]  # unchanged by rejected tables
        (tmp_path / "bad.json").write_text('{"device": "x"}')
        assert mlpgpu.lib().mlp_tuning_load(str(tmp_path / "bad.json").encode()) == 5
        mlpgpu.set_tuning_table([])
        assert mlpgpu.tuning_table() == []
    finally:
        mlpgpu.set_tuning_table(saved)


def test_argument_validation_needs_no_gpu(built_lib):
    """Malformed arguments are rejected with status codes and a message before
    any device call (MLP_ERR_ARG = 1, MLP_ERR_RANGE = 3)."""
    import ctypes as C

    import numpy as np

    import mlpgpu

    L = mlpgpu.lib()
    h = C.c_void_p()
    x = np.zeros(8, np.int32)
    for n in (-1, 0, 3, 4, 16384):
        assert L.mlp_problem_create_coords(n, x.ctypes.data, x.ctypes.data, 1, 1, C.byref(h)) == 3, n
        assert b"instance size out of range" in L.mlp_last_error()
    assert L.mlp_problem_create_coords(10, None, None, 1, 1, C.byref(h)) == 1
    assert L.mlp_last_error() == b"null argument"
    assert L.mlp_solver_create(None, 0, C.byref(h)) == 1
    assert L.mlp_batch_run(None, 31, 10) == 1
    assert L.mlp_server_create(0, 0, 0, C.byref(h)) == 1
    assert b"budget" in L.mlp_last_error()
