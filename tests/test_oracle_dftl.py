"""DFTL mode of the oracle (CPU): invariants, analytic cases, and how far
FP32 arithmetic drifts from FP64 in well-conditioned scenes.

DFTL mode (Mueller et al. 2012) has no counterpart in the reference shader,
so these checks come from the scheme itself: exact segment lengths after the
follow-the-leader projection, roots on their targets, a one-link pendulum
against its closed form, and the FP32/FP64 tolerances of DFTL mode
(one step <= 1e-5 x strand length, segment length <= 1e-5 relative, 60-frame
drift <= 1e-3 x strand length) in scenes where the physics does not amplify
rounding: strands swinging in the wind with 4 substeps, and light contacts.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import abi, scenarios
from tests import util


def run_both(spec, frames, dt=1 / 60):
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float32, lengths=spec.lengths)
    q, w = p.astype(np.float64), v.astype(np.float64)
    L = util.strand_lengths(p)
    hist = []
    for f in range(frames):
        t = (f + 1) * dt
        wind = scenarios.wind_at(t) if spec.wind else None
        oracle.frame(p, v, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=spec.spheres)
        oracle.frame(q, w, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=spec.spheres)
        hist.append((p.copy(), q.copy()))
    return L, hist


@pytest.mark.parametrize("n", [8, 16, 32])
def test_fp32_vs_fp64_well_conditioned(n):
    spec = util.hanging_spec(997, n, substeps=4)
    L, hist = run_both(spec, 60)
    p1, q1 = hist[0]
    assert util.max_pos_error_rel(p1, q1, L) <= 1e-5
    s32, s64 = util.segment_lengths(p1), util.segment_lengths(q1)
    assert np.max(np.abs(s32 - s64) / s64) <= 1e-5
    p60, q60 = hist[-1]
    assert util.max_pos_error_rel(p60, q60, L) <= 1e-3


@pytest.mark.parametrize("n", [8, 16])
def test_fp32_vs_fp64_one_step_with_contacts(n):
    spec = util.hanging_spec(997, n, substeps=4, spheres="side")
    L, hist = run_both(spec, 1)
    p1, q1 = hist[0]
    assert util.max_pos_error_rel(p1, q1, L) <= 1e-5


def test_segment_lengths_exact_without_contacts():
    spec = util.hanging_spec(200, 16, substeps=8)
    spec.sim.iterations = 1
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float64, lengths=spec.lengths)
    rest = p[:, 1:, 3].copy()
    for f in range(10):
        oracle.frame(p, v, spec.sim, 1 / 60, seed=7, wind=scenarios.wind_at((f + 1) / 60))
    np.testing.assert_allclose(util.segment_lengths(p), rest, rtol=1e-12)


def test_pendulum_single_substep_closed_form():
    """One link, one substep, no damping term at the tip: the tip goes to
    root + l * normalize(x + h v + h^2 g - root), velocity (p - x) / h."""
    roots = np.array([[0.0, 0.0, 0.0]], np.float32)
    normals = np.array([[1.0, 0.0, 0.0]], np.float32)
    sp = abi.strand_params(2, abi.HS_LENGTH_TOTAL, 0.5, 0.0, 0)
    sim = abi.sim_params_dftl(substeps=1, damping=0.9)
    p, v = oracle.init(roots, normals, sp, dtype=np.float64, lengths=np.array([0.5], np.float32))
    h = np.float64(np.float32(1 / 60))
    x = p[0, 1, :3].copy()
    oracle.frame(p, v, sim, float(np.float32(1 / 60)))
    g = np.array([0.0, np.float64(np.float32(-9.81)), 0.0])
    pred = x + h * h * g
    want = 0.5 * pred / np.linalg.norm(pred)
    np.testing.assert_allclose(p[0, 1, :3], want, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(v[0, 1, :3], (want - x) / h, rtol=1e-9)


def test_roots_reach_rigid_targets_at_frame_end():
    spec = scenarios.plain(ns=300, npoints=8)
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float64, lengths=spec.lengths)
    rest = p[:, 0, :3].astype(np.float32)
    for f in range(5):
        m = spec.transform((f + 1) / 60)
        tg = oracle.rigid_targets(rest, m, np.float64)
        oracle.frame(p, v, spec.sim, 1 / 60, spheres=spec.spheres_at((f + 1) / 60), root_targets=tg)
        np.testing.assert_allclose(p[:, 0, :3], tg, rtol=0, atol=1e-15)


def test_wind_jitter_is_per_strand_and_bounded():
    us = np.array([oracle.hash_u01(123, 2, i) for i in range(4096)])
    assert us.min() >= 0.0 and us.max() < 1.0
    assert abs(us.mean() - 0.5) < 0.02
    assert len(np.unique(us)) > 4000
    # Deterministic draws (pinned values of the counter hash).
    assert oracle.hash_u01(0, 1, 0) == oracle.hash_u01(0, 1, 0)
    assert oracle.hash_u01(0, 1, 0) != oracle.hash_u01(1, 1, 0)


def test_split_groom_matches_whole():
    """strand_base: a groom split in two halves hashes its strands like the
    whole groom, so the halves reproduce the whole bit for bit."""
    spec = scenarios.large(ns=2048, npoints=8)
    sp = spec.strand
    whole_p, whole_v = oracle.init(spec.roots, spec.normals, sp, dtype=np.float32, lengths=spec.lengths)
    halves = []
    for lo, hi in ((0, 1000), (1000, 2048)):
        sph = abi.strand_params(8, abi.HS_LENGTH_TOTAL, 0.5, 0.0, int(sp.seed), strand_base=lo)
        p, v = oracle.init(spec.roots[lo:hi], spec.normals[lo:hi], sph, dtype=np.float32,
                           lengths=spec.lengths[lo:hi])
        halves.append((lo, p, v))
    for f in range(3):
        w = scenarios.wind_at((f + 1) / 60)
        oracle.frame(whole_p, whole_v, spec.sim, 1 / 60, seed=int(sp.seed), wind=w, spheres=spec.spheres)
        for lo, p, v in halves:
            oracle.frame(p, v, spec.sim, 1 / 60, seed=int(sp.seed), wind=w, spheres=spec.spheres, strand_base=lo)
    util.assert_bit_equal(np.concatenate([h[1] for h in halves]), whole_p, "split positions")
    util.assert_bit_equal(np.concatenate([h[2] for h in halves]), whole_v, "split velocities")
