"""The C++ task API (include/mlp_gpu.hpp): it compiles against the C-ABI
library here; on a GPU the reference's own K2/K3/K4 test flow runs through it
(tests/cpp_task_api.cpp)."""
import json
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT

LIBDIR = os.path.join(ROOT, "wamca-gpu-mi_gb300", "lib")


def _build(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libmlpgpu.so")):
        import build_lib

        build_lib.build()
    exe = str(tmp_path / "cpp_task_api")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp_task_api.cpp"), "-L", LIBDIR, "-lmlpgpu", f"-Wl,-rpath,{LIBDIR}",
           "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert "warning" not in res.stderr, res.stderr
    return exe


def test_cpp_header_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_cpp_task_api_reference_known_answers(tmp_path, mlpgpu_mod):
    exe = _build(tmp_path)
    berlin = json.load(open(os.path.join(GOLDEN, "berlin52.json")))
    tsp = tmp_path / "berlin52.tsp"
    lines = ["NAME : berlin52", "TYPE : TSP", f"DIMENSION : {len(berlin['x'])}", "EDGE_WEIGHT_TYPE : EUC_2D",
             "NODE_COORD_SECTION"]
    lines += [f"{q + 1} {x} {y}" for q, (x, y) in enumerate(zip(berlin["x"], berlin["y"]))]
    lines.append("EOF")
    tsp.write_text("\n".join(lines) + "\n")
    res = subprocess.run([exe, str(tsp)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0 and res.stdout.strip().endswith("ok"), res.stdout + res.stderr
