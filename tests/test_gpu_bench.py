"""bench.py on the GPU, on small cases of the single-groom workloads: each
workload's setup (the groom, its per-frame inputs, the mapping query) runs
through the public API and the line carries the contract's keys."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload,strands", [("plain", 1024), ("large", 4096), ("skinned", 4096)])
def test_single_groom_line(built_library, workload, strands):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--workload", workload, "--strands",
                          str(strands), "--steps", "3", "--warmup", "3", "--e2e-steps", "2", "--no-cpu-baseline",
                          "--no-served", "--no-tess", "--no-others", "--no-alt-contract"],
                         capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, out.stdout
    line = json.loads(lines[0])
    assert line["config"]["workload"] == workload and line["config"]["strands"] == strands
    assert line["value"] > 0 and line["gpu_launches"] > 0
    assert line["mapping"] in ("a thread per strand", "lane groups (a lane per substep)")
    assert line["contract"].startswith("fast")
    for key in ("roofline", "e2e", "clocks"):
        assert key in line, key
    assert line["e2e"]["d2h_bytes_per_step"] == strands * line["config"]["points_per_strand"] * 12
    for e in (line["e2e"], line["e2e"]["xyzw"], line["e2e"]["synchronous"]):
        assert len(e["runs"]) == 3 and e["value"] == sorted(e["runs"])[1]  # the median run
