"""The merge's branch-free cross-neighbourhood conflict test (move_shape /
shapes_conflict, wamca-gpu-mi_gb300/csrc/mlp_common.cuh) equals the oracle's
canMerge restatement (mlkernel.cu:649-729) on every pair of moves of every
tour of size 6 .. 24 (tests/shape_conflict_check.cpp, compiled on the host)."""
import os
import subprocess

import oracle
from conftest import ROOT


def test_shapes_conflict_equals_can_merge(tmp_path):
    oracle.lib()  # builds oracle/liboracle.so when missing
    odir = os.path.dirname(oracle.LIB)
    exe = str(tmp_path / "shape_conflict_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "wamca-gpu-mi_gb300", "csrc"),
           os.path.join(ROOT, "tests", "shape_conflict_check.cpp"), "-L", odir, "-loracle", f"-Wl,-rpath,{odir}",
           "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip().endswith("0 mismatches"), run.stdout
