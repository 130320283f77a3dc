"""Skinned roots (HS_ROOT_SKINNED) on the GPU.

The step kernel skins each strand's rest root by dual-quaternion blending
at the start of the frame (the reference's skinning_DQBS,
src/shaders/shared/inc_skinning.glsl:54-82) and moves the root to it over
the substeps. Held to the FP32 oracle bit for bit: the oracle converts the
same skinning matrices, skins the same rest roots and runs the same frames.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu

DT = 1 / 60


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def make(ctx, spec):
    g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    g.set_skin(spec.bones, spec.weights)
    return g


def feed(g, spec, f, dual_quats=False):
    m = spec.rig.matrices(f + 1)
    if dual_quats:
        g.set_bone_dual_quats(oracle.matrix_to_dual_quat(m))
    else:
        g.set_bone_matrices(m)
    g.set_spheres(spec.spheres_at(f + 1))


@pytest.mark.parametrize("ns,n,nsph", [(4096, 16, 8), (700, 64, 32), (97, 8, 0)])
def test_skinned_bit_exact_vs_oracle(hs, ns, n, nsph):
    spec = scenarios.skinned(ns=ns, npoints=n, nspheres=nsph, substeps=4)
    sp = spec.strand
    p, v = oracle.init(spec.roots, spec.normals, sp, dtype=np.float32)
    with hs.Context() as ctx:
        g = make(ctx, spec)
        for f in range(12):
            feed(g, spec, f)
            g.update(DT)
            dq = oracle.matrix_to_dual_quat(spec.rig.matrices(f + 1))
            tg = oracle.skin_targets(spec.roots, spec.bones, spec.weights, dq, dtype=np.float32)
            oracle.frame(p, v, spec.sim, DT, seed=int(sp.seed), spheres=spec.spheres_at(f + 1), root_targets=tg)
            if f in (0, 11):
                util.assert_bit_equal(g.readback(), p, f"frame {f + 1} positions")
                util.assert_bit_equal(g.readback_velocities()[..., :3], v[..., :3], f"frame {f + 1} velocities")
        # The roots sit on their skinned targets at the end of each frame.
        np.testing.assert_array_equal(g.readback()[:, 0, :3], tg)


def test_dual_quats_and_matrices_agree_and_batch_matches_plain(hs):
    spec = scenarios.skinned(ns=2000, npoints=24, nspheres=12, substeps=8)
    other = scenarios.plain(ns=300, npoints=8)
    with hs.Context() as ctx:
        a = make(ctx, spec)
        b = make(ctx, spec)
        c = make(ctx, spec)
        o1 = ctx.groom(other.roots, other.normals, other.strand, other.sim)
        o2 = ctx.groom(other.roots, other.normals, other.strand, other.sim)
        for f in range(6):
            feed(a, spec, f)
            feed(b, spec, f, dual_quats=True)
            feed(c, spec, f)
            for o in (o1, o2):
                o.set_root_transform(other.transform((f + 1) * DT))
                o.set_spheres(other.spheres_at((f + 1) * DT))
            a.update(DT)
            o1.update(DT)
            ctx.update_many([b, o2], DT)
            ctx.update_many_noalloc([c], DT)
        util.assert_bit_equal(b.readback(), a.readback(), "batched / dual quaternions vs plain / matrices")
        util.assert_bit_equal(c.readback(), a.readback(), "no-alloc batched vs plain")
        util.assert_bit_equal(o2.readback(), o1.readback(), "rigid groom in the same batch")


def test_skin_errors(hs):
    spec = scenarios.skinned(ns=64, npoints=8, nspheres=0)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        with pytest.raises(hs.HairSimError) as e:
            g.update(DT)                                   # no influences yet
        assert e.value.status == abi.HS_ERR_NOT_INITIALIZED
        bad = spec.bones.copy()
        bad[0, 0] = abi.HS_MAX_BONES
        with pytest.raises(hs.HairSimError) as e:
            g.set_skin(bad, spec.weights)
        assert e.value.status == abi.HS_ERR_INVALID_ARG
        g.set_skin(spec.bones, spec.weights)               # uses bones 0..3
        g.set_bone_matrices(spec.rig.matrices(1)[:2])
        with pytest.raises(hs.HairSimError) as e:
            g.update(DT)                                   # palette too short
        assert e.value.status == abi.HS_ERR_NOT_INITIALIZED
        with pytest.raises(hs.HairSimError):
            g.set_bone_matrices(np.zeros((abi.HS_MAX_BONES + 1, 16), np.float32))
        with pytest.raises(hs.HairSimError):
            g.set_bone_dual_quats(np.zeros((1, 8), np.float32))  # zero rotation part
        g.set_bone_matrices(spec.rig.matrices(1))
        g.update(DT)


def test_skinned_full_size_sampled_parity(hs):
    """The whole skinned configuration (1,048,576 strands x 64 points, 32
    spheres, S = 8) on the GPU for 12 frames; the FP32 oracle re-runs
    sampled blocks of strands (strands are independent given their roots'
    skinned targets) and must agree bit for bit."""
    spec = scenarios.skinned()
    sp = spec.strand
    rng = np.random.default_rng(5)
    blocks = [(int(b), 128) for b in rng.choice(spec.nstrands - 128, size=6, replace=False)]
    with hs.Context() as ctx:
        g = make(ctx, spec)
        pos0, vel0 = g.readback(), g.readback_velocities()
        samp = [(pos0[b:b + k].copy(), vel0[b:b + k].copy()) for b, k in blocks]
        del pos0, vel0
        for f in range(12):
            feed(g, spec, f)
            g.update(DT)
            dq = oracle.matrix_to_dual_quat(spec.rig.matrices(f + 1))
            for (b, k), (p, v) in zip(blocks, samp):
                tg = oracle.skin_targets(spec.roots[b:b + k], spec.bones[b:b + k], spec.weights[b:b + k], dq,
                                         dtype=np.float32)
                oracle.frame(p, v, spec.sim, DT, seed=int(sp.seed), spheres=spec.spheres_at(f + 1),
                             root_targets=tg, strand_base=b)
        P, V = g.readback(), g.readback_velocities()
        for (b, k), (p, v) in zip(blocks, samp):
            util.assert_bit_equal(P[b:b + k], p, f"frame 12 strands {b}..{b + k}")
            util.assert_bit_equal(V[b:b + k, :, :3], v[..., :3], f"frame 12 strands {b}..{b + k} velocities")
        assert np.isfinite(P).all()


def test_gpu_skinned_roots_match_the_reference_shader(hs):
    """The step kernel's skinning, pinned directly: a groom rooted at the
    golden rest points, skinned by the golden palette for one frame, ends
    the frame with its roots on the reference shader's skinned points
    (tests/golden/ref_skin.npz, inc_skinning.glsl compiled as C++), bit for
    bit."""
    g = util.load_golden("skin")
    n = len(g["rest"])
    normals = np.tile(np.array([[0.0, 1.0, 0.0]], np.float32), (n, 1))
    sp = abi.strand_params(4, abi.HS_LENGTH_TOTAL, 0.3, 0.0, 3)
    sim = abi.sim_params_dftl(substeps=2, root_mode=abi.HS_ROOT_SKINNED)
    with hs.Context() as ctx:
        gr = ctx.groom(g["rest"], normals, sp, sim)
        gr.set_skin(g["bones"], g["weights"])
        gr.set_bone_dual_quats(g["dq"])
        gr.update(DT)
        util.assert_bit_equal(gr.readback()[:, 0, :3], g["out"], "skinned roots vs the reference shader")
