"""bench.py --impl reference on the CPU: the reference arm times the oracle's
FP32 restatement of the step on the host cores and prints one JSON line
with the keys the benchmark contract asks for, on the same workload
configuration as the GPU arm."""
from __future__ import annotations

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_reference(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                         capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    line = run_reference("--workload", "plain", "--steps", "2", "--warmup", "1")
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "contract", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["metric"] == line["unit"] == "strand-point substeps/s"
    assert line["higher_is_better"] is True
    assert line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["contract"].startswith("exact")


def test_reference_arm_config_is_the_gpu_arms():
    """The workload description is the one the GPU arm prints (the
    arithmetic contract is reported beside it, not in it)."""
    sys.path.insert(0, ROOT)
    import bench
    line = run_reference("--workload", "plain", "--steps", "1", "--warmup", "0")
    for contract in ("exact", "fast"):
        assert line["config"] == bench.make_workload("plain", None, contract).config(1)


def test_reference_arm_other_ranks_print_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "plain",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, cwd=ROOT, env=env,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
