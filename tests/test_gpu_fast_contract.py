"""The FAST arithmetic contract (hs_contract) on the GPU.

FAST takes the DFTL step's reciprocal square roots (the chain link's and
the sphere push-out normal's) from the GPU's instruction (PTX rsqrt.approx)
instead of the EXACT contract's fixed sequence of rounded operations. The CPU cannot repeat that instruction bit
for bit, so FAST frames are held
  * to the DFTL tolerances against the FP64 oracle on the benchmark
    configurations, with the coverage the EXACT contract is held to
    (tests/test_gpu_tolerances.py);
  * to a bound against the EXACT contract's FP32 oracle: after one frame,
    FAST_VS_EXACT x strand length on the strands the one-step tolerance
    covers (no contact, well-conditioned);
and, within one GPU, to themselves: every kernel form (batched or per
groom, a thread or a lane group per strand) gives the same bits.
"""
from __future__ import annotations

import numpy as np
import pytest

from barbu_gb300 import abi, scenarios
from tests import tolerance as T
from tests import util

pytestmark = pytest.mark.gpu

FRAMES, MID = 60, 31
KEEP = (1, MID - 1, MID, FRAMES)
FAST_VS_EXACT = 5e-6  # x strand length, one frame, strands without contact in it, well-conditioned


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def fast(sim):
    s = abi.SimParams.from_buffer_copy(sim)
    s.contract = abi.HS_CONTRACT_FAST
    return s


def sample(groom, blk):
    P, V = groom.readback(), groom.readback_velocities()
    return np.concatenate([np.concatenate([P[b:b + k], V[b:b + k]], axis=-1) for b, k in blk])


def make(ctx, spec, sim):
    g = ctx.groom(spec.roots, spec.normals, spec.strand, sim, lengths=spec.lengths)
    if isinstance(spec, scenarios.SkinnedSpec):
        g.set_skin(spec.bones, spec.weights)
    return g


def check_against_exact(feed, blk, states, report):
    """One frame from the initial state: FAST against the EXACT contract's
    FP32 oracle, on the strands without contact in that frame and not
    ill-conditioned in it (the strands the one-step tolerance covers)."""
    ref = T.oracle_states(feed, blk, 1, 1)
    L = util.strand_lengths(states[0][..., :4])
    err = np.linalg.norm(states[1][..., :3].astype(np.float64) - ref[1][..., :3], axis=-1).max(axis=1) / L
    free = ~report.contact_step & ~report.step_ill
    assert free.any()
    assert err[free].max() <= FAST_VS_EXACT, (err[free].max(), float(free.mean()))
    return float(err[free].max())


def single_groom(hs, spec, blk):
    sim = fast(spec.sim)
    feed = T.Feed(spec)
    with hs.Context() as ctx:
        g = make(ctx, spec, sim)
        states = {0: sample(g, blk)}
        for f in range(FRAMES):
            feed.gpu(g, f)
            g.update(T.DT)
            if f + 1 in KEEP:
                states[f + 1] = sample(g, blk)
    r = T.evaluate(feed, blk, states, FRAMES, MID)
    dev = check_against_exact(feed, blk, states, r)
    return r, dev


def test_fast_contract_only_in_dftl_mode(hs):
    spec = scenarios.plain(ns=64, npoints=8)
    with hs.Context() as ctx:
        ref = abi.sim_params_reference(1.45)
        ref.contract = abi.HS_CONTRACT_FAST
        with pytest.raises(hs.HairSimError) as e:
            ctx.groom(spec.roots, spec.normals, spec.strand, ref)
        assert e.value.status == abi.HS_ERR_INVALID_ARG
        bad = abi.sim_params_dftl()
        bad.contract = 2
        with pytest.raises(hs.HairSimError):
            ctx.groom(spec.roots, spec.normals, spec.strand, bad)


def test_fast_plain_config(hs):
    spec = scenarios.plain()
    r, dev = single_groom(hs, spec, [(0, spec.nstrands)])
    print("plain fast", r.summary(), "vs exact", dev)
    r.check(min_covered=0.05, min_step_covered=0.3)


def test_fast_large_config(hs):
    spec = scenarios.large()
    r, dev = single_groom(hs, spec, T.blocks(spec.nstrands, 16, 256))
    print("large fast", r.summary(), "vs exact", dev)
    r.check(min_covered=0.8, min_step_covered=0.85)


def test_fast_skinned_config(hs):
    spec = scenarios.skinned()
    r, dev = single_groom(hs, spec, T.blocks(spec.nstrands, 4, 128))
    print("skinned fast", r.summary(), "vs exact", dev)
    r.check(min_covered=0.15, min_step_covered=0.8)


def test_fast_batched_config(hs):
    """The 64-groom batched workload under FAST through hs_update_many."""
    specs = scenarios.batched()
    picks = (0, 17, 33, 63)
    blks = {gi: T.blocks(specs[gi].nstrands, 4, 128) for gi in picks}
    feeds = [T.Feed(s) for s in specs]
    with hs.Context() as ctx:
        grooms = [make(ctx, s, fast(s.sim)) for s in specs]
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
        r = T.evaluate(feeds[gi], blks[gi], states[gi], FRAMES, MID)
        dev = check_against_exact(feeds[gi], blks[gi], states[gi], r)
        print(f"batched fast groom {gi}", r.summary(), "vs exact", dev)
        reports.append(r)
    cat = lambda name: np.concatenate([getattr(r, name) for r in reports])  # noqa: E731
    allr = T.Report(**{f: cat(f) for f in T.Report.__dataclass_fields__})
    allr.check(min_covered=0.4, min_step_covered=0.7)


def test_fast_frames_agree_across_kernel_forms(hs):
    """Batched (mixed contracts in one batch) and per-groom updates, a
    thread or a lane group per strand: the same bits under each contract."""
    specs = scenarios.batched(ngrooms=6, scale=0.02)
    specs.append(scenarios.plain(ns=500, npoints=6))   # register form (N <= 8)
    sims = [fast(s.sim) if i % 2 == 0 else s.sim for i, s in enumerate(specs)]

    def run(ctx, batched, mapping):
        gs = [make(ctx, s, sim) for s, sim in zip(specs, sims)]
        for g in gs:
            g.set_mapping(mapping)
        for f in range(5):
            t = (f + 1) * T.DT
            for g, s in zip(gs, specs):
                m = s.transform(t)
                if m is not None:
                    g.set_root_transform(m)
                g.set_spheres(s.spheres_at(t))
            if batched:
                ctx.update_many(gs, T.DT)
            else:
                for g in gs:
                    g.update(T.DT)
        out = [(g.readback(), g.readback_velocities()) for g in gs]
        for g in gs:
            g.destroy()
        return out

    with hs.Context() as ctx:
        want = run(ctx, False, abi.HS_MAPPING_THREAD)
        for batched, mapping in ((True, abi.HS_MAPPING_THREAD), (False, abi.HS_MAPPING_LANES)):
            got = run(ctx, batched, mapping)
            for k, ((p, v), (pw, vw)) in enumerate(zip(got, want)):
                util.assert_bit_equal(p, pw, f"groom {k} positions (batched={batched}, mapping={mapping})")
                util.assert_bit_equal(v, vw, f"groom {k} velocities (batched={batched}, mapping={mapping})")
        # FAST and EXACT differ (the contract is in effect), within the bound.
        exact = [make(ctx, s, s.sim) for s in specs[:1]]
        f0 = [make(ctx, s, fast(s.sim)) for s in specs[:1]]
        for g in exact + f0:
            g.set_root_transform(specs[0].transform(T.DT))
            g.set_spheres(specs[0].spheres_at(T.DT))
            g.update(T.DT)
        a, b = exact[0].readback(), f0[0].readback()
        assert not np.array_equal(a, b)
        L = util.strand_lengths(a)
        assert (np.linalg.norm(a[..., :3] - b[..., :3], axis=-1).max(axis=1) / L).max() <= 1e-4
