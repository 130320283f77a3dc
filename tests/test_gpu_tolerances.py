"""The benchmark configurations against the FP64 oracle, on the GPU.

Each configuration runs whole on the GPU for 60 frames (the batched one
through hs_update_many, as benchmarked); sampled blocks of strands are
re-run by the oracle: in FP32 (the library's arithmetic contract: bit for
bit) and in FP64 (Mueller et al.'s algorithm as written), from the same
initial state and inputs. The DFTL tolerances are asserted on the
strands tests/tolerance.py says they can hold for, and the fraction of
strands each bound covers is asserted with it:
  * one frame (from the initial state, and from the GPU's state of frame
    30): position error <= 1e-5 x strand length and segment-length error
    <= 1e-5 relative, on strands without contact and not ill-conditioned in
    that frame; <= 1e-3 x strand length on every strand;
  * 60 frames: drift <= 1e-3 x strand length on contact-free,
    well-conditioned strands.
Every configuration is also run for the frames it is specified with (plain
600, large and batched 300, skinned 1,000; the skinned one under both
arithmetic contracts): EXACT bit for bit with the FP32 oracle at the last
frame, the one-frame bounds, and the drift bound on 99 % of the strands
that stay contact-free and well-conditioned over the run (ten times it on
all of them: tolerance.Report.check_long).
"""
from __future__ import annotations

import numpy as np
import pytest

from barbu_gb300 import scenarios
from tests import tolerance as T
from tests import util

pytestmark = pytest.mark.gpu

FRAMES, MID = 60, 31
KEEP = (1, MID - 1, MID, FRAMES)


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def sample(groom, blk):
    P, V = groom.readback(), groom.readback_velocities()
    return np.concatenate([np.concatenate([P[b:b + k], V[b:b + k]], axis=-1) for b, k in blk])


def make(ctx, spec):
    g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    if isinstance(spec, scenarios.SkinnedSpec):
        g.set_skin(spec.bones, spec.weights)
    return g


def check_against_fp32_oracle(feed, blk, states, frames=FRAMES):
    ref = T.oracle_states(feed, blk, frames, MID)
    for f in (1, MID, frames):
        util.assert_bit_equal(states[f][..., :4], ref[f][..., :4], f"frame {f} positions vs FP32 oracle")
        util.assert_bit_equal(states[f][..., 4:7], ref[f][..., 4:7], f"frame {f} velocities vs FP32 oracle")


def single_groom(hs, spec, blk, frames=FRAMES, exact=True):
    """The whole groom on the GPU for `frames` frames; the sampled blocks
    against the FP32 oracle (EXACT contract: bit for bit) and the FP64
    oracle."""
    feed = T.Feed(spec)
    keep = (1, MID - 1, MID, frames)
    with hs.Context() as ctx:
        g = make(ctx, spec)
        states = {0: sample(g, blk)}
        for f in range(frames):
            feed.gpu(g, f)
            g.update(T.DT)
            if f + 1 in keep:
                states[f + 1] = sample(g, blk)
    if exact:
        check_against_fp32_oracle(feed, blk, states, frames)
    return T.evaluate(feed, blk, states, frames, MID)


def test_plain_config_fp64_tolerances(hs):
    """4,096 x 16, S = 4, one moving sphere r = 1 on which the roots sit:
    88 % of the strands fall onto it (contact)."""
    spec = scenarios.plain()
    r = single_groom(hs, spec, [(0, spec.nstrands)])
    print("plain", r.summary())
    r.check(min_covered=0.05, min_step_covered=0.3)


def test_large_config_fp64_tolerances(hs):
    """262,144 x 32, S = 8, 16 spheres, wind: the benchmarked single groom."""
    spec = scenarios.large()
    blk = T.blocks(spec.nstrands, 16, 256)
    r = single_groom(hs, spec, blk)
    print("large", r.summary())
    r.check(min_covered=0.8, min_step_covered=0.85)


def test_skinned_config_fp64_tolerances(hs):
    """1,048,576 x 64 on the skinned cylinder, S = 8, 32 spheres riding on
    the bones: three quarters of the strands touch a sphere."""
    spec = scenarios.skinned()
    blk = T.blocks(spec.nstrands, 4, 128)
    r = single_groom(hs, spec, blk)
    print("skinned", r.summary())
    r.check(min_covered=0.15, min_step_covered=0.8)


@pytest.mark.parametrize("contract", ["exact", "fast"])
def test_skinned_config_1000_frames(hs, contract):
    """The skinned configuration's own length: 1,000 frames (bone rotations
    are random walks, so the rig keeps moving)."""
    from barbu_gb300 import abi
    spec = scenarios.skinned()
    if contract == "fast":
        spec.sim.contract = abi.HS_CONTRACT_FAST
    blk = T.blocks(spec.nstrands, 4, 128)
    r = single_groom(hs, spec, blk, frames=1000, exact=contract == "exact")
    print(f"skinned, 1,000 frames, {contract}", r.summary(), r.long_run())
    r.check_long(min_covered=0.05, min_step_covered=0.8)


def test_plain_config_600_frames(hs):
    spec = scenarios.plain()
    r = single_groom(hs, spec, [(0, spec.nstrands)], frames=600)
    print("plain, 600 frames", r.summary(), r.long_run())
    r.check_long(min_covered=0.02, min_step_covered=0.3)


def test_large_config_300_frames(hs):
    spec = scenarios.large()
    r = single_groom(hs, spec, T.blocks(spec.nstrands, 16, 256), frames=300)
    print("large, 300 frames", r.summary(), r.long_run())
    r.check_long(min_covered=0.8, min_step_covered=0.85)


def test_batched_config_300_frames(hs):
    """The batched workload's 300 frames through hs_update_many."""
    specs = scenarios.batched()
    picks = (0, 5, 17, 33, 50, 63)
    frames = 300
    keep = (1, MID - 1, MID, frames)
    blks = {gi: T.blocks(specs[gi].nstrands, 4, 128) for gi in picks}
    feeds = [T.Feed(s) for s in specs]
    with hs.Context() as ctx:
        grooms = [make(ctx, s) for s in specs]
        states = {gi: {0: sample(grooms[gi], blks[gi])} for gi in picks}
        for f in range(frames):
            for g, fd in zip(grooms, feeds):
                fd.gpu(g, f)
            ctx.update_many(grooms, T.DT)
            if f + 1 in keep:
                for gi in picks:
                    states[gi][f + 1] = sample(grooms[gi], blks[gi])
    reports = []
    for gi in picks:
        check_against_fp32_oracle(feeds[gi], blks[gi], states[gi], frames)
        reports.append(T.evaluate(feeds[gi], blks[gi], states[gi], frames, MID))
    cat = lambda name: np.concatenate([getattr(r, name) for r in reports])
    allr = T.Report(**{f: cat(f) for f in T.Report.__dataclass_fields__})
    print("batched, 300 frames", allr.summary(), allr.long_run())
    allr.check_long(min_covered=0.3, min_step_covered=0.7)


def test_batched_config_fp64_tolerances(hs):
    """The 64-groom batched workload through hs_update_many (one graph per
    frame, the benchmarked path); six grooms of every point count sampled."""
    specs = scenarios.batched()
    picks = (0, 5, 17, 33, 50, 63)
    blks = {gi: T.blocks(specs[gi].nstrands, 4, 128) for gi in picks}
    feeds = [T.Feed(s) for s in specs]
    with hs.Context() as ctx:
        grooms = [make(ctx, s) for s in specs]
        states = {gi: {0: sample(grooms[gi], blks[gi])} for gi in picks}
        for f in range(FRAMES):
            for g, fd in zip(grooms, feeds):
                fd.gpu(g, f)
            ctx.update_many(grooms, T.DT)
            if f + 1 in KEEP:
                for gi in picks:
                    states[gi][f + 1] = sample(grooms[gi], blks[gi])
    reports = []
    for gi in picks:
        check_against_fp32_oracle(feeds[gi], blks[gi], states[gi])
        r = T.evaluate(feeds[gi], blks[gi], states[gi], FRAMES, MID)
        print(f"batched groom {gi} (N = {specs[gi].npoints})", r.summary())
        reports.append(r)
    cat = lambda name: np.concatenate([getattr(r, name) for r in reports])
    allr = T.Report(**{f: cat(f) for f in T.Report.__dataclass_fields__})
    print("batched, sampled grooms together", allr.summary())
    allr.check(min_covered=0.4, min_step_covered=0.7)
