"""The benchmark configurations' FP32 arithmetic against FP64 (CPU).

The FP32 oracle is the library's arithmetic contract (the GPU equals it bit
for bit, tests/test_gpu_tolerances.py), so the DFTL tolerances can be
checked here on sampled strands of every configuration without a GPU; see
tests/tolerance.py for which strands each bound covers. Also: DFTL's segment
form is the same algorithm as the world-coordinate form (FP64 runs of both
agree to rounding), and in FP32 it drifts far less.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import scenarios
from tests import tolerance as T
from tests import util

FRAMES, MID = 60, 31


def run(spec, blk):
    feed = T.Feed(spec)
    return T.evaluate(feed, blk, T.oracle_states(feed, blk, FRAMES, MID), FRAMES, MID)


def test_plain_config():
    spec = scenarios.plain()
    run(spec, [(0, spec.nstrands)]).check(min_covered=0.05, min_step_covered=0.3)


def test_large_config_sample():
    spec = scenarios.large()
    run(spec, T.blocks(spec.nstrands, 6, 128)).check(min_covered=0.7, min_step_covered=0.8)


@pytest.mark.parametrize("gi", [5, 17, 63])
def test_batched_config_grooms(gi):
    spec = scenarios.batched()[gi]
    run(spec, T.blocks(spec.nstrands, 2, 128)).check(min_covered=0.3, min_step_covered=0.6)


def test_skinned_config_sample():
    spec = scenarios.skinned(ns=65536)
    run(spec, T.blocks(spec.nstrands, 3, 128)).check(min_covered=0.02, min_step_covered=0.7)


def _run_form(spec, idx, dtype, form, frames):
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float32, lengths=spec.lengths)
    p = np.ascontiguousarray(p[idx], dtype=dtype)
    v = np.ascontiguousarray(v[idx], dtype=dtype)
    for f in range(frames):
        t = (f + 1) / 60
        oracle.frame(p, v, spec.sim, 1 / 60, seed=int(spec.strand.seed), wind=scenarios.wind_at(t),
                     strand_base=int(idx[0]), form=form)
    return p


def test_segment_form_is_the_same_algorithm():
    """FP64, hanging strands swinging in the wind: both forms agree to
    rounding over 30 frames of S = 8."""
    spec = util.hanging_spec(256, 24, substeps=8)
    idx = np.arange(256)
    a = _run_form(spec, idx, np.float64, oracle.FORM_WORLD, 30)
    b = _run_form(spec, idx, np.float64, oracle.FORM_SEGMENT, 30)
    L = util.strand_lengths(a)
    assert util.max_pos_error_rel(a, b, L) <= 1e-11


def test_segment_form_drifts_less_in_fp32():
    """Large configuration's geometry without spheres, S = 8, 60 frames:
    the segment form's FP32 drift from FP64 is at least 20x smaller than
    the world form's (median over strands) and under 1e-4 x length where
    the strand is not upright."""
    spec = scenarios.large()
    idx = np.arange(4096, 4096 + 512)
    ref = _run_form(spec, idx, np.float64, oracle.FORM_WORLD, 60)
    seg = _run_form(spec, idx, np.float32, oracle.FORM_SEGMENT, 60)
    world = _run_form(spec, idx, np.float32, oracle.FORM_WORLD, 60)
    L = util.strand_lengths(ref)
    e = lambda p: np.linalg.norm(p[..., :3].astype(np.float64) - ref[..., :3], axis=-1).max(axis=1) / L
    es, ew = e(seg), e(world)
    assert np.median(ew) >= 20 * np.median(es), (np.median(ew), np.median(es))
    tilted = spec.normals[idx, 1] < 0.9
    assert es[tilted].max() <= 1e-4, es[tilted].max()


def test_checker_catches_planted_mistakes():
    """The tolerance check has teeth: FP32 oracle states pass it, and the
    same states with one point of one covered strand moved by three times
    a bound (one step after frame 1, drift after the last frame) fail it."""
    spec = scenarios.large()
    blk = T.blocks(spec.nstrands, 2, 64)
    feed = T.Feed(spec)
    frames, mid = 12, 7
    states = T.oracle_states(feed, blk, frames, mid)
    rep = T.evaluate(feed, blk, states, frames, mid)
    rep.check(min_covered=0.5)
    free = ~rep.contact_step & ~rep.step_ill & ~rep.contact & ~rep.ill
    assert free.any()
    s = int(np.flatnonzero(free)[0])
    for f, size in ((1, 3 * T.ONE_STEP_TOL), (frames, 3 * T.DRIFT_TOL)):
        bad = {k: v.copy() for k, v in states.items()}
        bad[f][s, -1, 0] += np.float32(size * rep.lengths[s])
        with pytest.raises(AssertionError):
            T.evaluate(feed, blk, bad, frames, mid).check(min_covered=0.5)
