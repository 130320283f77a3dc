"""Oracle: the tessellation stream pass (CPU).

Known answers of the reference's tessellation evaluation
(src/shaders/hair/02_tess_stream/tes_stream_hair.glsl): hermite_mix
(inc_maths.glsl:210-228) passes through the segment's two control points
at u = 0 and u = 1, so the ends of each interpolated strand segment are the
triangle's points blended with the random barycentric coordinates
(sample_triangle2, :107-115, which folds coordinates beyond the diagonal
back into the triangle); the relative position is smoothstep2 of
j/N + u/N (:65-66). The output has 2 vertices per line segment, in the
order [instance][triangle][segment][line][subsegment].
"""
from __future__ import annotations

import numpy as np

import oracle
from barbu_gb300 import abi


def setup(ns=5, n=4, nf=3, seed=1):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (ns, n, 4)).astype(np.float32)
    tan = rng.uniform(-0.2, 0.2, (ns, n, 4)).astype(np.float32)
    faces = rng.integers(0, ns, (nf, 3)).astype(np.uint32)
    rand = rng.random(abi.HS_TESS_RANDOM_SIZE).astype(np.float32)
    return pos, tan, faces, rand


def smoothstep2(x):
    t = min(max(x, 0.0), 1.0)
    return t * t * t * (10 + t * (-15 + 6 * t))


def bary(rx, ry):
    sx, sy = rx, ry
    if sx + sy > 1.0:
        sx = max(sx, sy)
        sy = min(sx, sy)
        sx = 1.0 - sx
    return sx, sy, 1.0 - (sx + sy)


def test_segment_ends_are_the_blended_control_points():
    pos, tan, faces, rand = setup()
    ninst, nlines, nsub = 2, 3, 4
    out = oracle.tess(pos, tan, faces, rand, ninst, nlines, nsub, 1.45).reshape(ninst, len(faces), 3, nlines, nsub,
                                                                                2, 4)
    for inst in range(ninst):
        for f, (a, b, c) in enumerate(faces):
            for j in range(3):
                for line in range(nlines):
                    r = int(np.float32(line / nlines) * np.float32(40) + inst) % abi.HS_TESS_RANDOM_SIZE
                    cx, cy, cz = bary(float(rand[4 * r]), float(rand[4 * r + 1]))
                    start = out[inst, f, j, line, 0, 0]
                    end = out[inst, f, j, line, nsub - 1, 1]
                    for k in range(3):
                        want0 = cx * pos[a, j, k] + cy * pos[b, j, k] + cz * pos[c, j, k]
                        want1 = cx * pos[a, j + 1, k] + cy * pos[b, j + 1, k] + cz * pos[c, j + 1, k]
                        assert abs(start[k] - want0) < 1e-5 and abs(end[k] - want1) < 1e-5
                    assert abs(start[3] - smoothstep2(j / 4)) < 1e-6
                    assert abs(end[3] - smoothstep2(j / 4 + 1 / 4)) < 1e-6
                    # Consecutive segments share their joint.
                    seg = out[inst, f, j, line]
                    np.testing.assert_array_equal(seg[1:, 0], seg[:-1, 1])


def test_barycentric_fold_keeps_points_in_the_triangle():
    pos, tan, faces, rand = setup(ns=3, n=2, nf=1)
    pos[:, :, :3] = 0
    pos[0, :, 0] = 1  # triangle (1,0,0), (0,1,0), (0,0,1) at both points
    pos[1, :, 1] = 1
    pos[2, :, 2] = 1
    tan[:] = 0
    faces[:] = [[0, 1, 2]]
    for seed in range(20):
        rand = np.random.default_rng(seed).random(abi.HS_TESS_RANDOM_SIZE).astype(np.float32)
        out = oracle.tess(pos, tan, faces, rand, 16, 16, 1, 1.0)
        xyz = out[:, :3].astype(np.float64)
        assert (xyz >= -1e-7).all() and np.abs(xyz.sum(axis=1) - 1).max() < 1e-6


def test_counts_and_tangent_scale():
    pos, tan, faces, rand = setup(ns=4, n=6, nf=5)
    a = oracle.tess(pos, tan, faces, rand, 3, 2, 16, 1.0)
    assert a.shape == (2 * 3 * 5 * 5 * 2 * 16, 4)
    b = oracle.tess(pos, tan * np.float32(2), faces, rand, 3, 2, 16, 0.5)
    np.testing.assert_array_equal(a, b)  # tangent * scale is what enters
    assert np.isfinite(a).all()


def load_tess_golden():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_tess.npz"))


def test_oracle_matches_reference_shader_golden_vectors():
    """ref_tess.npz holds the reference's own tessellation evaluation shader
    (compiled as C++) on the scalp after 60 frames, with the scalp's
    triangles: the restatement matches it bit for bit."""
    g = load_tess_golden()
    for case in ("a", "b"):
        ninst, nlines, nsub, scale = g[f"params_{case}"]
        out = oracle.tess(g["pos"], g["tangents"], g[f"faces_{case}"], g["random"], int(ninst), int(nlines),
                          int(nsub), float(scale))
        np.testing.assert_array_equal(out.view(np.uint32), g[f"out_{case}"].view(np.uint32))


def test_oracle_matches_reference_shader_live():
    """Where the reference tree is present, the same against the shader
    compiled now, on other inputs."""
    import pytest
    if not oracle.ref_tes_available():
        pytest.skip("reference shader library not built here")
    pos, tan, faces, rand = setup(ns=40, n=4, nf=25, seed=9)
    for params in ((3, 2, 16, 1.45), (16, 16, 2, 0.3), (1, 7, 5, 1.0)):
        a = oracle.tess(pos, tan, faces, rand, *params)
        b = oracle.ref_tes_stream(pos, tan, faces, rand, *params)
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
