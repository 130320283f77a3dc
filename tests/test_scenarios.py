"""The seeded benchmark grooms have the shapes the benchmark configurations
state (CPU): strand and point counts, substeps, sphere counts and radii,
length ranges, and where the roots lie (the large groom's on the faces of a
subdivision-5 icosphere, the skinned groom's on the 448 quads of its
cylinder, root k on face or quad floor(k * faces / strands))."""
from __future__ import annotations

import math

import numpy as np

from barbu_gb300 import abi, scenarios


def test_plain_groom():
    s = scenarios.plain()
    assert (s.nstrands, s.npoints, s.sim.substeps) == (4096, 16, 4)
    np.testing.assert_allclose(np.linalg.norm(s.roots.astype(np.float64), axis=1), 1.0, atol=1e-6)
    assert np.array_equal(s.roots, s.normals)
    assert s.spheres.tolist() == [[0.0, 0.0, 0.0, 1.0]]
    assert s.moving_roots == "translate_x" and s.amp == 0.2
    assert s.sim.mode == abi.HS_MODE_DFTL


def test_large_groom_roots_on_icosphere_faces():
    s = scenarios.large()
    ns = s.nstrands
    assert (ns, s.npoints, s.sim.substeps) == (262144, 32, 8)
    assert s.lengths.min() >= 0.3 and s.lengths.max() <= 0.8
    assert s.spheres.shape == (16, 4)
    assert (s.spheres[:, 3] >= 0.1).all() and (s.spheres[:, 3] <= 0.4).all()
    d = np.linalg.norm(s.spheres[:, :3].astype(np.float64), axis=1)
    assert (d >= 1.0 - 1e-6).all() and (d <= 1.6 + 1e-6).all()
    n = s.normals.astype(np.float64)
    np.testing.assert_allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    assert np.abs(s.roots - s.normals).max() <= 0.05 + 1e-6  # hash noise of amplitude 0.05
    V, F = scenarios.icosphere(5)
    assert (len(V), len(F)) == (10242, 20480)
    face = (np.arange(ns) * len(F)) // ns
    # The normal is the projection of a point of its face: a non-negative
    # combination of the face's three vertices.
    M = np.stack([V[F[face, 0]], V[F[face, 1]], V[F[face, 2]]], axis=2)
    coef = np.linalg.solve(M, n[:, :, None])[..., 0]
    assert coef.min() >= -1e-5
    assert s.wind and s.sim.wind_jitter == np.float32(0.2)


def test_batched_grooms():
    specs = scenarios.batched()
    assert len(specs) == 64
    ns = np.array([s.nstrands for s in specs])
    assert ns.min() >= 1024 and ns.max() <= 131072
    assert int(ns.sum()) == 1_806_729
    assert sum(s.nstrands * s.npoints for s in specs) == 34_961_424
    assert {s.npoints for s in specs} <= {8, 16, 24, 32}
    for s in specs:
        assert s.sim.substeps == 8 and s.sim.root_mode == abi.HS_ROOT_RIGID
        assert 1 <= len(s.spheres) <= 16
        assert 0.0 <= s.omega_deg <= 30.0 and s.amp == 0.3
        assert s.lengths.min() >= 0.3 and s.lengths.max() <= 0.8


def test_skinned_groom_roots_on_cylinder_quads():
    s = scenarios.skinned()
    ns = s.nstrands
    assert (ns, s.npoints, s.sim.substeps) == (1048576, 64, 8)
    assert s.sim.root_mode == abi.HS_ROOT_SKINNED
    r = s.roots.astype(np.float64)
    np.testing.assert_allclose(np.hypot(r[:, 0], r[:, 2]), 0.5, atol=1e-6)
    assert r[:, 1].min() >= 0.0 and r[:, 1].max() <= 2.0 + 1e-6
    quad = (np.arange(ns) * 448) // ns
    theta = np.mod(np.arctan2(r[:, 2], r[:, 0]), 2 * math.pi)
    seg = np.floor(theta / (2 * math.pi / 64)).astype(np.int64)
    ring = np.floor(r[:, 1] / (2.0 / 7)).astype(np.int64)
    # float32 rounding may move a root sitting on a quad edge to its neighbour
    assert np.mean(ring * 64 + seg != quad) < 1e-4
    # Two influences: the heavier bone in slot 0 (and 1, 2 at weight 0), the other in slot 3.
    assert (s.bones[:, 0] == s.bones[:, 1]).all() and (s.bones[:, 0] == s.bones[:, 2]).all()
    assert (np.abs(s.bones[:, 0].astype(int) - s.bones[:, 3].astype(int)) == 1).all()
    assert (s.weights[:, 1:] == 0).all()
    assert s.weights[:, 0].min() >= 0.5 and s.weights[:, 0].max() <= 1.0
    assert len(s.sphere_rest) == 32
    assert (s.sphere_rest[:, 3] >= 0.1).all() and (s.sphere_rest[:, 3] <= 0.25).all()
