"""Stored strand order (GPU).

A groom stores its strands in a Z-order of their roots, whatever order the
caller passes them in, so that the 32 strands of a warp are neighbours
(the per-warp sphere culling and instruction stream then do not depend on
the caller's order). Every input and output of the API stays in the
caller's order: a groom given its strands shuffled must give, strand for
strand, the bit-identical frames of the same groom given them in order,
and keep_order (stored as given) must too.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu

DT = 1 / 60


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def strand(spec, keep=False, jitter=None):
    s = spec.strand
    return abi.strand_params(int(s.points_per_strand), int(s.length_rule), float(s.max_length),
                             float(s.length_jitter if jitter is None else jitter), int(s.seed), int(s.strand_base),
                             keep_order=keep)


def shuffled(a, perm):
    return None if a is None else np.ascontiguousarray(np.asarray(a)[perm])


@pytest.mark.parametrize("jitter", [False, True])
def test_shuffled_rigid_groom_matches_ordered(hs, jitter):
    """Per-strand length and wind jitter hash the caller's strand index: with
    jitter, the shuffled groom stored in Z-order must match the same
    shuffled groom stored as given; without, also the ordered groom."""
    spec = scenarios.plain(ns=3000, npoints=16)
    perm = np.random.default_rng(3).permutation(spec.nstrands)
    sim = abi.SimParams.from_buffer_copy(spec.sim)
    sim.wind_jitter = 0.2 if jitter else 0.0
    lj = 0.1 if jitter else 0.0
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, strand(spec, jitter=lj), sim)
        b = ctx.groom(spec.roots[perm], spec.normals[perm], strand(spec, jitter=lj), sim)
        c = ctx.groom(spec.roots[perm], spec.normals[perm], strand(spec, keep=True, jitter=lj), sim)
        order = b.strand_order()
        assert np.array_equal(np.sort(order), np.arange(spec.nstrands))
        assert not np.array_equal(order, np.arange(spec.nstrands))
        assert np.array_equal(c.strand_order(), np.arange(spec.nstrands))
        for f in range(12):
            t = (f + 1) * DT
            for g in (a, b, c):
                g.set_root_transform(spec.transform(t))
                g.set_spheres(spec.spheres_at(t))
                g.set_wind(scenarios.wind_at(t))
            ctx.update_many([a, b], DT)
            c.update(DT)
        pc, vc = c.readback(), c.readback_velocities()
        util.assert_bit_equal(b.readback(), pc, "z-ordered positions")
        util.assert_bit_equal(b.readback_velocities(), vc, "z-ordered velocities")
        util.assert_bit_equal(b.readback_xyz(), pc[..., :3], "z-ordered xyz")
        if not jitter:
            util.assert_bit_equal(pc, a.readback()[perm], "shuffled vs ordered positions")
            util.assert_bit_equal(vc, a.readback_velocities()[perm], "shuffled vs ordered velocities")
        for g in (a, b, c):
            g.destroy()


class _Dev:
    """A device buffer as a torch tensor, from a raw pointer."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": "<f4", "data": (ptr, False), "version": 3}


def test_device_columns_follow_the_stored_order(hs):
    spec = scenarios.plain(ns=1000, npoints=8)
    perm = np.random.default_rng(4).permutation(spec.nstrands)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots[perm], spec.normals[perm], strand(spec), spec.sim)
        g.set_spheres(spec.spheres)
        g.set_root_transform(spec.transform(DT))
        g.update(DT)
        ctx.sync()
        want = g.readback()
        ptr, lay = g.device_positions()
        dev = torch.as_tensor(_Dev(ptr, (lay.points_per_strand, lay.strand_stride, 4)), device="cuda").cpu().numpy()
        order = g.strand_order()
        # column j of [point][strand] is the caller's strand order[j]
        util.assert_bit_equal(dev[:, :lay.nstrands].transpose(1, 0, 2), want[order], "device columns")
        # both export layouts come back in the caller's order
        n = spec.nstrands * spec.npoints * 4
        buf = torch.empty(n, dtype=torch.float32, device="cuda")
        g.export(buf.data_ptr(), n, abi.HS_EXPORT_STRAND_MAJOR)
        ctx.sync()
        util.assert_bit_equal(buf.cpu().numpy().reshape(want.shape), want, "strand-major export")
        g.export(buf.data_ptr(), n, abi.HS_EXPORT_POINT_MAJOR)
        ctx.sync()
        util.assert_bit_equal(buf.cpu().numpy().reshape(spec.npoints, spec.nstrands, 4).transpose(1, 0, 2), want,
                              "point-major export")
        g.destroy()


def test_shuffled_explicit_roots_and_state_init(hs):
    spec = scenarios.plain(ns=700, npoints=8)
    perm = np.random.default_rng(5).permutation(spec.nstrands)
    sim = abi.SimParams.from_buffer_copy(spec.sim)
    sim.root_mode = abi.HS_ROOT_EXPLICIT
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, strand(spec), sim)
        b = ctx.groom(spec.roots[perm], spec.normals[perm], strand(spec), sim)
        for f in range(6):
            tgt = (spec.roots + np.float32(0.01 * (f + 1))).astype(np.float32)
            a.set_roots(tgt)
            b.set_roots(tgt[perm])
            a.update(DT)
            b.update(DT)
        pa, va = a.readback(), a.readback_velocities()
        util.assert_bit_equal(b.readback(), pa[perm], "explicit roots")
        # A groom set up from a shuffled state, advanced a frame.
        c = ctx.groom_from_state(pa[perm], va[perm], sim, seed=int(spec.strand.seed))
        d = ctx.groom_from_state(pa, va, sim, seed=int(spec.strand.seed))
        util.assert_bit_equal(c.readback(), pa[perm], "state round trip")
        for g, t in ((c, (spec.roots + np.float32(0.08))[perm]), (d, spec.roots + np.float32(0.08))):
            g.set_roots(t.astype(np.float32))
            g.update(DT)
        util.assert_bit_equal(c.readback(), d.readback()[perm], "frame after a shuffled state")
        for g in (a, b, c, d):
            g.destroy()


def test_shuffled_skinned_groom_matches_ordered(hs):
    spec = scenarios.skinned(ns=2000, npoints=16, nspheres=8, substeps=2)
    perm = np.random.default_rng(6).permutation(spec.nstrands)
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, strand(spec), spec.sim, lengths=spec.lengths)
        a.set_skin(spec.bones, spec.weights)
        b = ctx.groom(spec.roots[perm], spec.normals[perm], strand(spec), spec.sim,
                      lengths=shuffled(spec.lengths, perm))
        b.set_skin(spec.bones[perm], spec.weights[perm])
        for f in range(6):
            for g in (a, b):
                g.set_bone_matrices(spec.rig.matrices(f + 1))
                g.set_spheres(spec.spheres_at(f + 1))
                g.update(DT)
        util.assert_bit_equal(b.readback(), a.readback()[perm], "skinned positions")
        a.destroy()
        b.destroy()


def test_shuffled_tessellation_matches_ordered(hs):
    spatial = pytest.importorskip("scipy.spatial")
    spec = scenarios.plain(ns=300, npoints=8)
    perm = np.random.default_rng(8).permutation(spec.nstrands)
    inv = np.argsort(perm)
    faces = spatial.ConvexHull(spec.roots.astype(np.float64)).simplices.astype(np.uint32)
    rng = np.random.default_rng(9)
    tangents = rng.uniform(-0.1, 0.1, (spec.nstrands, spec.npoints, 4)).astype(np.float32)
    rand = rng.random(abi.HS_TESS_RANDOM_SIZE).astype(np.float32)
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, strand(spec), spec.sim)
        b = ctx.groom(spec.roots[perm], spec.normals[perm], strand(spec), spec.sim)
        for f in range(3):
            for g in (a, b):
                g.set_root_transform(spec.transform((f + 1) * DT))
                g.set_spheres(spec.spheres)
                g.update(DT)
        a.tess_setup(faces, tangents, rand)
        b.tess_setup(inv[faces].astype(np.uint32), tangents[perm], rand)  # the same triangles, shuffled names
        a.tess_stream()
        b.tess_stream()
        util.assert_bit_equal(b.tess_readback(), a.tess_readback(), "tessellated vertices")
        a.destroy()
        b.destroy()


def test_shuffled_served_request_matches_ordered(hs):
    spec = scenarios.plain(ns=1500, npoints=8)
    perm = np.random.default_rng(10).permutation(spec.nstrands)
    with hs.Context() as ctx, hs.Server(ctx, budget_bytes=64 << 20) as srv:
        ta = srv.submit(spec.roots, spec.normals, strand(spec), spec.sim, frames=5, spheres=spec.spheres,
                        wind=(0.5, 0.0, 0.2), keep=True)
        tb = srv.submit(spec.roots[perm], spec.normals[perm], strand(spec), spec.sim, frames=5,
                        spheres=spec.spheres, wind=(0.5, 0.0, 0.2), keep=True)
        for _ in range(8):
            srv.tick(DT)
        pa, va = srv.collect(ta)
        pb, vb = srv.collect(tb)
        util.assert_bit_equal(pb, pa[perm], "served positions")
        util.assert_bit_equal(vb, va[perm], "served velocities")
