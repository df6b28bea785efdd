"""The device constructor's restatement of the reference's candidate sort
(wamca-gpu-mi_gb300/csrc/mlp_refsort.cuh, compiled here for the host) gives
the C++ library's std::sort permutation on tie-heavy inputs, in both orders,
including its heap-sort fallback and the constructor's repeated re-sorts of
one array (tests/refsort_check.cpp)."""
import os
import subprocess

from conftest import ROOT


def test_refsort_equals_library_sort(tmp_path):
    exe = str(tmp_path / "refsort_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "wamca-gpu-mi_gb300", "csrc"),
           os.path.join(ROOT, "tests", "refsort_check.cpp"), "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip().endswith(" 0 mismatches"), run.stdout
