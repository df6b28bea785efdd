"""bench.py's reference arm (the oracle port of the reference's CPU path,
timed on the host cores) prints one JSON line with the keys of the bench
contract; it needs no GPU, so the line is checked here on the CPU."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_plain_launch_count_matches_the_loop_modes():
    # The gpu_launches claim of a plain step: prepare, statistics reset, then
    # passes of 16 iterations of (sweep, merge), each with the while node's
    # condition kernel in the device-side loop (the default) and without it in
    # host-checked graph replays.
    sys.path.insert(0, ROOT)
    import bench

    assert bench.plain_launches(259) == 2 + 33 * 17
    assert bench.plain_launches(259, device_loop=False) == 2 + 32 * 17
    assert bench.plain_launches(16) == 2 + 33 and bench.plain_launches(17) == 2 + 66
    assert bench.plain_launches(0) == bench.plain_launches(1) == 2 + 33
