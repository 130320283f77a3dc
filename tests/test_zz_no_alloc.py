"""hs_update_many_noalloc on the GPU: the batched update without allocation.

Its scratch (tile counters, bucket directory, groom table) lives in one
fixed device array shared by every call, so two calls in a row must both
match hs_update_many bit for bit: the second finds the first's contents in
the array and must clear what has to start at zero. Collected last, and
self-contained, so it passes alone in a fresh process and after the rest.
"""
from __future__ import annotations

import pytest

from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu

DT = 1 / 60


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def specs():
    """Uneven strand and point counts, both modes and both DFTL contracts,
    every bucket size class."""
    out = scenarios.batched(ngrooms=7, scale=0.02)  # N in {8, 16, 24, 32}
    g = util.load_golden("scalp")                     # reference mode, N = 4
    sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.1, int(g["strand_seed"]))
    out.append(scenarios.GroomSpec(g["roots"], g["normals"], sp, abi.sim_params_reference(1.45), None,
                                   g["bspheres"][0][None].copy()))
    out.append(scenarios.plain(ns=33, npoints=5))     # one full warp + 1 strand
    out.append(scenarios.large(ns=700, npoints=48, nspheres=6))  # 64-point class
    for s in (scenarios.plain(ns=500, npoints=12), scenarios.plain(ns=90, npoints=6)):
        s.sim.contract = abi.HS_CONTRACT_FAST             # the FAST contract's own buckets
        out.append(s)
    return out


def set_inputs(gr, spec, f):
    t = (f + 1) * DT
    m = spec.transform(t)
    if m is not None:
        gr.set_root_transform(m)
    if spec.wind:
        gr.set_wind(scenarios.wind_at(t))
    gr.set_spheres(spec.spheres_at(t))


def test_noalloc_matches_update_many_on_two_calls(hs):
    ss = specs()
    with hs.Context() as ctx:
        ref = [ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths) for s in ss]
        got = [ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths) for s in ss]
        for f in range(2):
            for a, b, s in zip(ref, got, ss):
                set_inputs(a, s, f)
                set_inputs(b, s, f)
            ctx.update_many(ref, DT)
            ctx.update_many_noalloc(got, DT)
            for k, (a, b) in enumerate(zip(ref, got)):
                util.assert_bit_equal(b.readback(), a.readback(), f"call {f + 1}, groom {k}: positions")
                util.assert_bit_equal(b.readback_velocities(), a.readback_velocities(),
                                      f"call {f + 1}, groom {k}: velocities")


def test_noalloc_rejects_lists_beyond_its_maximum(hs):
    s = scenarios.plain(ns=64, npoints=8)
    with hs.Context() as ctx:
        gr = ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths)
        too_many = [gr] * (abi.HS_NOALLOC_MAX_GROOMS + 1)
        with pytest.raises(hs.HairSimError) as e:
            ctx.update_many_noalloc(too_many, DT)
        assert e.value.status == abi.HS_ERR_INVALID_ARG
        assert "maximum" in str(e.value)
