"""The committed ncu summaries the bench line reads: one per workload and
contract, each naming its command, carrying the two figures bench.py
reads (DRAM bytes and warp instructions per frame), and captured at the
kernel sources in the tree (their hash), so that the bench line's traffic
and issue figures describe the kernels it runs."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

WORKLOADS = ["batched", "large", "plain", "skinned"]
ALGORITHMIC_BYTES = {  # 64 B per point per frame
    "batched": 64 * 34_961_424,
    "large": 64 * 262_144 * 32,
    "plain": 64 * 4_096 * 16,
    "skinned": 64 * 1_048_576 * 64,
}


@pytest.mark.parametrize("contract", ["", "_fast"])
@pytest.mark.parametrize("workload", WORKLOADS)
def test_profile_is_current(workload, contract):
    import bench
    name = workload + contract
    text = open(os.path.join(ROOT, "profiles", f"step_{name}.md")).read()
    assert "ncu " in text and "--clock-control none" in text and "python bench.py" in text
    captured, current = bench.profile_meta(name)
    assert current, f"step_{name}.md captured at {captured}, sources at {bench.csrc_hash()}"
    traffic = bench.profiled_value(name, "traffic_bytes_per_frame")
    inst = bench.profiled_value(name, "warp_instructions_per_frame")
    assert traffic is not None and inst is not None and inst > 0
    if workload != "plain":  # the plain groom's state stays in the L2 between frames
        assert 0.8 < traffic / ALGORITHMIC_BYTES[workload] < 1.05
