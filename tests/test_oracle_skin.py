"""Oracle: dual-quaternion skinning of roots (CPU).

The reference skins mesh vertices with dual-quaternion blending
(src/shaders/shared/inc_skinning.glsl:22-82) but has no tests; these are
known-answer checks from the algebra (Kavan et al. 2008): a unit dual
quaternion applies its rigid motion exactly, blending one bone is that
bone's motion, a quaternion and its negation are the same rotation, and a
first weight <= 1e-6 switches skinning off (:23-25). The matrix to dual
quaternion conversion is checked on each of its four branches.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from tests import util
from barbu_gb300 import abi, scenarios


def rot(axis, deg):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    x, y, z = a
    c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def rigid(axis, deg, t):
    M = np.eye(4)
    M[:3, :3] = rot(axis, deg)
    M[:3, 3] = t
    return M


def colmajor(M):
    return M.T.astype(np.float32).reshape(16)


def points(n=64, seed=3):
    return np.random.default_rng(seed).uniform(-1, 1, (n, 3)).astype(np.float32)


def one_bone(n):
    return np.zeros((n, 4), np.uint8), np.tile(np.array([[1, 0, 0]], np.float32), (n, 1))


@pytest.mark.parametrize("axis,deg", [((1, 0, 0), 40), ((0, 1, 0), 179), ((1, 0, 0), 179), ((0, 0, 1), 179),
                                      ((1, 2, 3), 75), ((0, 1, 0), 0)])
def test_matrix_to_dual_quat_is_the_rigid_motion(axis, deg):
    """Every branch of the conversion (trace > 0, and each largest diagonal)."""
    M = rigid(axis, deg, (0.3, -1.2, 2.0))
    dq = oracle.matrix_to_dual_quat(colmajor(M))[0]
    assert abs(np.dot(dq[:4], dq[:4]) - 1.0) < 1e-6
    assert abs(np.dot(dq[:4], dq[4:])) < 1e-6  # unit dual quaternion: real . dual = 0
    p = points()
    b, w = one_bone(len(p))
    got = oracle.skin_targets(p, b, w, dq[None], dtype=np.float64)
    want = (M @ np.c_[p.astype(np.float64), np.ones(len(p))].T).T[:, :3]
    assert np.abs(got - want).max() < 2e-6


def test_identity_palette_keeps_rest_roots():
    p = points()
    dq = np.array([[0, 0, 0, 1, 0, 0, 0, 0]] * 2, np.float32)
    b = np.tile(np.array([[0, 1, 1, 0]], np.uint8), (len(p), 1))
    w = np.tile(np.array([[0.3, 0.2, 0.1]], np.float32), (len(p), 1))
    for dt in (np.float32, np.float64):
        np.testing.assert_array_equal(oracle.skin_targets(p, b, w, dq, dtype=dt), p.astype(dt))


def test_first_weight_below_epsilon_switches_skinning_off():
    p = points()
    dq = oracle.matrix_to_dual_quat(colmajor(rigid((0, 1, 0), 30, (1, 2, 3))))
    b, w = one_bone(len(p))
    w[:, 0] = 1e-6
    np.testing.assert_array_equal(oracle.skin_targets(p, b, w, dq, dtype=np.float32), p)


def test_negated_quaternion_blends_the_same():
    """sign(dot(real[b3], real[bk])) flips antipodal bones (:65)."""
    p = points()
    m0 = colmajor(rigid((0, 0, 1), 20, (0.1, 0, 0)))
    m1 = colmajor(rigid((0, 0, 1), 35, (0.0, 0.2, 0)))
    dq = oracle.matrix_to_dual_quat(np.stack([m0, m1]))
    flipped = dq.copy()
    flipped[0] = -flipped[0]
    b = np.tile(np.array([[0, 0, 0, 1]], np.uint8), (len(p), 1))
    w = np.tile(np.array([[0.6, 0, 0]], np.float32), (len(p), 1))
    a = oracle.skin_targets(p, b, w, dq, dtype=np.float64)
    c = oracle.skin_targets(p, b, w, flipped, dtype=np.float64)
    assert np.abs(a - c).max() < 1e-6


def test_blend_of_equal_bones_is_that_bone_and_float_tracks_double():
    p = points(256)
    M = colmajor(rigid((1, 1, 0), 50, (0.5, 0.5, -0.5)))
    dq = oracle.matrix_to_dual_quat(np.stack([M, M]))
    b = np.tile(np.array([[0, 1, 1, 1]], np.uint8), (len(p), 1))
    w = np.random.default_rng(1).dirichlet([1, 1, 1, 1], len(p))[:, :3].astype(np.float32)
    one = oracle.skin_targets(p, *one_bone(len(p)), dq[:1], dtype=np.float64)
    mix64 = oracle.skin_targets(p, b, w, dq, dtype=np.float64)
    mix32 = oracle.skin_targets(p, b, w, dq, dtype=np.float32)
    assert np.abs(mix64 - one).max() < 2e-6
    assert np.abs(mix32 - mix64).max() < 4e-6


def test_cylinder_rig_moves_at_most_two_degrees_a_frame():
    rig = scenarios.SkinRig(7)
    prev = rig.angles(0)
    for f in range(1, 200):
        a = rig.angles(f)
        assert np.linalg.norm(a - prev, axis=1).max() <= math.radians(2.0) + 1e-12
        assert np.linalg.norm(a, axis=1).max() <= math.radians(25.0) + 1e-12
        prev = a


def test_skinned_drift_fp32_vs_fp64_within_tolerance():
    """60 frames of a small skinned cylinder (no contacts, bones walking at
    most 0.5 deg a frame): the FP32 instantiation (which the GPU matches bit
    for bit) stays within 1e-3 x strand length of FP64. Faster rigs amplify
    FP32 rounding further (the velocity is a difference of positions over
    the substep); that drift is measured, not bounded, here."""
    spec = scenarios.skinned(ns=256, npoints=16, nspheres=0, substeps=4)
    spec.rig = scenarios.SkinRig(spec.rig.seed, step_deg=0.5, clamp_deg=10.0)
    sp = spec.strand
    p32, v32 = oracle.init(spec.roots, spec.normals, sp, dtype=np.float32)
    p64, v64 = oracle.init(spec.roots, spec.normals, sp, dtype=np.float64)
    dt = 1 / 60
    for f in range(60):
        dq = oracle.matrix_to_dual_quat(spec.rig.matrices(f + 1))
        t32 = oracle.skin_targets(spec.roots, spec.bones, spec.weights, dq, dtype=np.float32)
        t64 = oracle.skin_targets(spec.roots, spec.bones, spec.weights, dq, dtype=np.float64)
        oracle.frame(p32, v32, spec.sim, dt, seed=int(sp.seed), root_targets=t32)
        oracle.frame(p64, v64, spec.sim, dt, seed=int(sp.seed), root_targets=t64)
    err = np.abs(p32[..., :3].astype(np.float64) - p64[..., :3]).max()
    assert err <= 1e-3 * float(sp.max_length), err
    assert np.abs(p32[:, 0, :3] - spec.roots).max() > 1e-3  # the roots did move
    assert abi.HS_ROOT_SKINNED == spec.sim.root_mode


def test_oracle_matches_the_reference_skinning_shader():
    """Pinned: the oracle's skinning equals the reference's own
    inc_skinning.glsl (apply_skinning + skinning_DQBS compiled as C++ by
    oracle/ref_glsl/make_ref.py; tests/golden/ref_skin.npz) bit for bit,
    edge cases included (first weight 0 or Epsilon(), an antipodal bone)."""
    g = util.load_golden("skin")
    got = oracle.skin_targets(g["rest"], g["bones"], g["weights"], g["dq"], dtype=np.float32)
    util.assert_bit_equal(got, g["out"], "skinned points vs the reference shader")
    if oracle.ref_skin_available():  # where the reference tree was compiled
        util.assert_bit_equal(oracle.ref_skin(g["rest"], g["bones"], g["weights"], g["dq"]), g["out"],
                              "reference shader rebuilt")
