"""Batched update (hs_update_many) and the autotuner (GPU).

A groom advanced in a batch must come out bit-identical to the same groom
advanced alone with hs_update: a strand's frame depends only on its own
state and its groom's constants, whatever else shares the launch.
"""
from __future__ import annotations

import pytest

from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def mixed_specs():
    """Grooms of uneven strand counts, point counts and modes."""
    specs = scenarios.batched(ngrooms=7, scale=0.02)  # 20 .. 2,600 strands, N in {8,16,24,32}
    g = util.load_golden("scalp")                      # reference mode, N = 4
    sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.1, int(g["strand_seed"]))
    specs.append(scenarios.GroomSpec(g["roots"], g["normals"], sp, abi.sim_params_reference(1.45), None,
                                     g["bspheres"][0][None].copy()))
    odd = scenarios.plain(ns=33, npoints=5)            # 33 strands: one full warp + 1
    specs.append(odd)
    return specs


def set_inputs(gr, spec, f, dt=1 / 60):
    t = (f + 1) * dt
    m = spec.transform(t)
    if m is not None:
        gr.set_root_transform(m)
    if spec.wind:
        gr.set_wind(scenarios.wind_at(t))
    gr.set_spheres(spec.spheres_at(t))


def make(ctx, specs):
    return [ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths) for s in specs]


def test_update_many_bit_identical_to_plain(hs):
    specs = mixed_specs()
    with hs.Context() as ctx:
        alone = make(ctx, specs)
        mixed = make(ctx, specs)
        for f in range(20):
            for gr, s in zip(alone, specs):
                set_inputs(gr, s, f)
                gr.update(1 / 60)
            for gr, s in zip(mixed, specs):
                set_inputs(gr, s, f)
            ctx.update_many(mixed, 1 / 60)
            if f in (0, 1, 19):
                for a, b in zip(alone, mixed):
                    util.assert_bit_equal(b.readback(), a.readback(), f"frame {f + 1} positions")
                    util.assert_bit_equal(b.readback_velocities(), a.readback_velocities(), f"frame {f + 1} velocities")


def test_full_size_batched_workload_bit_identical_to_plain(hs):
    """The whole batched configuration (64 grooms, 1.8 M strands, N 8-32,
    S = 8, rigid roots, 1-16 spheres): autotuned hs_update_many against one
    hs_update per groom, every state word after 3 frames."""
    specs = scenarios.batched()
    with hs.Context() as ctx:
        alone = make(ctx, specs)
        mixed = make(ctx, specs)
        for gr, s in zip(mixed, specs):
            set_inputs(gr, s, 0)
        ctx.autotune(mixed, 1 / 60)  # restores the state it advances
        for f in range(3):
            for gr, s in zip(alone, specs):
                set_inputs(gr, s, f)
                gr.update(1 / 60)
            for gr, s in zip(mixed, specs):
                set_inputs(gr, s, f)
            ctx.update_many(mixed, 1 / 60)
        for k, (a, b) in enumerate(zip(alone, mixed)):
            util.assert_bit_equal(b.readback(), a.readback(), f"groom {k} positions")
            util.assert_bit_equal(b.readback_velocities(), a.readback_velocities(), f"groom {k} velocities")


def test_autotune_restores_state_and_keeps_results(hs):
    specs = mixed_specs()
    with hs.Context() as ctx:
        alone = make(ctx, specs)
        mixed = make(ctx, specs)
        for gr, s in zip(mixed, specs):
            set_inputs(gr, s, 0)
        before = [gr.readback() for gr in mixed]
        assert ctx.tune_entries() == []
        trials = ctx.autotune(mixed, 1 / 60)
        assert trials > 0
        chosen = ctx.tune_entries()
        assert chosen and all(e["ms"] > 0 and e["variant"] in (0, 1, 2, 6, 7)
                              and e["warps_per_block"] in (1, 2, 4, 8, 16) for e in chosen)
        for gr, b in zip(mixed, before):
            util.assert_bit_equal(gr.readback(), b, "state after autotune")
        for f in range(5):
            for gr, s in zip(alone, specs):
                set_inputs(gr, s, f)
                gr.update(1 / 60)
            for gr, s in zip(mixed, specs):
                set_inputs(gr, s, f)
            ctx.update_many(mixed, 1 / 60)
        for a, b in zip(alone, mixed):
            util.assert_bit_equal(b.readback(), a.readback(), "after tuned frames")


def test_update_many_follows_set_changes(hs):
    specs = mixed_specs()
    with hs.Context() as ctx:
        alone = make(ctx, specs)
        mixed = make(ctx, specs)
        active = list(range(len(specs)))
        for f in range(12):
            if f == 4:
                active = active[2:]          # two grooms leave
            if f == 8:
                active = [0, 1] + active     # and come back
            for i in active:
                set_inputs(alone[i], specs[i], f)
                alone[i].update(1 / 60)
                set_inputs(mixed[i], specs[i], f)
            ctx.update_many([mixed[i] for i in active], 1 / 60)
        for a, b in zip(alone, mixed):
            util.assert_bit_equal(b.readback(), a.readback(), "after set changes")


def test_update_many_rejects_bad_lists(hs):
    with hs.Context() as ctx, hs.Context() as other:
        s = scenarios.plain(ns=64, npoints=8)
        a = ctx.groom(s.roots, s.normals, s.strand, s.sim)
        b = other.groom(s.roots, s.normals, s.strand, s.sim)
        with pytest.raises(hs.HairSimError):
            ctx.update_many([a, a], 1 / 60)
        with pytest.raises(hs.HairSimError):
            ctx.update_many([a, b], 1 / 60)
        ctx.update_many([], 1 / 60)


@pytest.mark.parametrize("variant,wpb", [(abi.HS_VARIANT_REGISTERS, 1), (abi.HS_VARIANT_REGISTERS_SHARED, 2),
                                         (abi.HS_VARIANT_STREAM, 4), (abi.HS_VARIANT_STREAM, 8),
                                         (abi.HS_VARIANT_STREAM, 1), (abi.HS_VARIANT_STREAM_TMEM, 4),
                                         (abi.HS_VARIANT_STREAM_TMEM, 8), (abi.HS_VARIANT_LANES, 8),
                                         (abi.HS_VARIANT_LANES, 16)])
def test_every_variant_matches_plain(hs, variant, wpb):
    specs = mixed_specs()
    specs.append(make_long_spec())
    with hs.Context() as ctx:
        for s in specs:
            for mode in (abi.HS_MODE_REFERENCE, abi.HS_MODE_DFTL):
                if s.npoints > 8 and variant < abi.HS_VARIANT_STREAM:
                    continue
                if variant == abi.HS_VARIANT_LANES and mode == abi.HS_MODE_REFERENCE:
                    continue  # lane groups run DFTL frames only
                w = wpb
                while True:
                    try:
                        ctx.tune_override(s.npoints, mode, variant, w, 1)
                        break
                    except hs.HairSimError:
                        w //= 2
                        if w == 0:
                            raise
        alone = make(ctx, specs)
        mixed = make(ctx, specs)
        for f in range(6):
            for gr, s in zip(alone, specs):
                set_inputs(gr, s, f)
                gr.update(1 / 60)
            for gr, s in zip(mixed, specs):
                set_inputs(gr, s, f)
            ctx.update_many(mixed, 1 / 60)
        for a, b in zip(alone, mixed):
            util.assert_bit_equal(b.readback(), a.readback(), f"variant {variant} positions")
            util.assert_bit_equal(b.readback_velocities(), a.readback_velocities(), f"variant {variant} velocities")


def make_long_spec():
    s = scenarios.large(ns=700, npoints=64, nspheres=8)
    return s


def test_unbuilt_variants_are_rejected(hs):
    """Register variants exist up to 8 points; variants 3-5 are not built."""
    with hs.Context() as ctx:
        for v in (3, 4, 5):
            with pytest.raises(hs.HairSimError):
                ctx.tune_override(16, abi.HS_MODE_DFTL, v, 1, 1)
        for n in (16, 32, 64):
            with pytest.raises(hs.HairSimError):
                ctx.tune_override(n, abi.HS_MODE_DFTL, abi.HS_VARIANT_REGISTERS, 1, 1)
        ctx.tune_override(8, abi.HS_MODE_DFTL, abi.HS_VARIANT_REGISTERS, 1, 1)
        # Lane groups: DFTL only; 16 warps per block is theirs alone.
        with pytest.raises(hs.HairSimError):
            ctx.tune_override(16, abi.HS_MODE_REFERENCE, abi.HS_VARIANT_LANES, 8, 1)
        with pytest.raises(hs.HairSimError):
            ctx.tune_override(16, abi.HS_MODE_DFTL, abi.HS_VARIANT_STREAM, 16, 1)
        ctx.tune_override(16, abi.HS_MODE_DFTL, abi.HS_VARIANT_LANES, 16, 1)


def test_pin_of_a_short_class_is_honoured_in_a_mixed_set(hs):
    """DFTL grooms of up to 32 points share one flat bucket unless their
    point class is pinned: a pin on the 8-point class gives those grooms a
    bucket of their own with the pinned shape (one more launch per frame),
    and the frames stay bit-identical to one update per groom."""
    specs = []
    for n, ns in ((8, 300), (16, 200), (32, 150)):
        s = scenarios.plain(ns=ns, npoints=n, seed=40 + n)
        specs.append(s)
    with hs.Context() as ctx:
        alone = make(ctx, specs)
        mixed = make(ctx, specs)

        def frame(f):
            for gr, s in zip(alone, specs):
                set_inputs(gr, s, f)
                gr.update(1 / 60)
            for gr, s in zip(mixed, specs):
                set_inputs(gr, s, f)
            before = ctx.launch_count()
            ctx.update_many(mixed, 1 / 60)
            return ctx.launch_count() - before

        assert frame(0) == 1  # one flat bucket
        ctx.tune_override(8, abi.HS_MODE_DFTL, abi.HS_VARIANT_REGISTERS, 2, 1)
        assert frame(1) == 2  # the pinned 8-point class runs apart
        assert frame(2) == 2
        for a, b in zip(alone, mixed):
            util.assert_bit_equal(b.readback(), a.readback(), "positions")
            util.assert_bit_equal(b.readback_velocities(), a.readback_velocities(), "velocities")
