"""bench.py's roofline arithmetic on the CPU: the HBM peak (measured, else
the stated fallback, saying which), the issue bound from the committed ncu
instruction count at the sampled clock, and the L2 note of each workload."""
from __future__ import annotations

import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_hbm_peak_measured_or_fallback(tmp_path, monkeypatch):
    import bench
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_hbm_peak() == (bench.HBM_FALLBACK_GBS, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6769.1}))
    assert bench.measured_hbm_peak() == (6769.1, "measured")


def test_issue_bound_arithmetic():
    import bench
    inst = bench.profiled_value("batched_fast", "warp_instructions_per_frame")
    r = bench.issue_roofline("batched_fast", 0.88, {"sm_mhz": 2070.0}, 152)
    assert r["warp_instructions_per_frame"] == inst
    assert r["peak"] == pytest.approx(4 * 152 * 2070e6)
    assert r["achieved"] == pytest.approx(inst / 0.88e-3)
    assert r["frac"] == pytest.approx(inst / 0.88e-3 / (4 * 152 * 2070e6))
    assert bench.issue_roofline("batched_fast", 0.88, {}, 152) is None  # no clock sample, no bound


def test_l2_notes():
    import bench
    assert bench.l2_note(4096 * 16).startswith("L2-resident")
    assert "exceeds the 129 MB L2" in bench.l2_note(34_961_424)
