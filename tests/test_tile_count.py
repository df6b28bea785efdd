"""The sweep tile-count helpers shared by the engine's tile lists, the serving
loop and the allocation-free evaluation (wamca-gpu-mi_gb300/csrc/mlp_common.cuh)
equal a direct enumeration of the tiles for every tour size up to 2048 and
every compiled tile shape, and the tiles cover each position pair once
(tests/tile_count_check.cpp, compiled on the host)."""
import os
import subprocess

from conftest import ROOT


def _cuda_include() -> str:
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return ""


def test_tile_counts_equal_enumeration(tmp_path):
    inc = _cuda_include()
    exe = str(tmp_path / "tile_count_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "wamca-gpu-mi_gb300", "csrc")]
    if inc:
        cmd += ["-I", inc]
    cmd += [os.path.join(ROOT, "tests", "tile_count_check.cpp"), "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip().endswith(" 0 mismatches"), run.stdout
