"""Tessellation stream pass (hs_tess_*) on the GPU, bit for bit against the
oracle's restatement of the reference's vs/tcs/tes/gs stream shaders
(src/shaders/hair/02_tess_stream/), on simulated positions."""
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


def hull_faces(roots):
    spatial = pytest.importorskip("scipy.spatial")
    return spatial.ConvexHull(roots.astype(np.float64)).simplices.astype(np.uint32)


def inputs(ns, n, seed):
    rng = np.random.default_rng(seed)
    tangents = rng.uniform(-0.1, 0.1, (ns, n, 4)).astype(np.float32)
    rand = rng.random(abi.HS_TESS_RANDOM_SIZE).astype(np.float32)
    return tangents, rand


@pytest.mark.parametrize("ns,n,frames,params", [(300, 8, 5, (3, 2, 16, 1.45)), (64, 32, 2, (2, 5, 7, 1.0)),
                                                (448, 4, 3, (1, 16, 16, 1.45))])
def test_tess_bit_exact_vs_oracle(hs, ns, n, frames, params):
    spec = scenarios.plain(ns=ns, npoints=n)
    faces = hull_faces(spec.roots)
    tangents, rand = inputs(ns, n, ns + n)
    p = abi.TessParams(*params)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        g.set_spheres(spec.spheres)
        for f in range(frames):
            g.set_root_transform(spec.transform((f + 1) * DT))
            g.update(DT)
        g.tess_setup(faces, tangents, rand)
        count = g.tess_stream(p)
        got = g.tess_readback()
        pos = g.readback()
    want = oracle.tess(pos, tangents, faces, rand, *params)
    assert count == want.shape[0] == 2 * params[0] * len(faces) * (n - 1) * params[1] * params[2]
    util.assert_bit_equal(got, want, "tessellated vertices")


def test_tess_errors(hs):
    spec = scenarios.plain(ns=40, npoints=8)
    tangents, rand = inputs(40, 8, 3)
    faces = np.array([[0, 1, 2], [3, 4, 5]], np.uint32)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        with pytest.raises(hs.HairSimError) as e:
            g.tess_stream()
        assert e.value.status == abi.HS_ERR_NOT_INITIALIZED
        with pytest.raises(hs.HairSimError):
            g.tess_setup(np.array([[0, 1, 40]], np.uint32), tangents, rand)    # strand out of range
        with pytest.raises(hs.HairSimError):
            g.tess_setup(faces, tangents, rand[:100])                          # wrong random size
        g.tess_setup(faces, tangents, rand)
        for bad in ((0, 2, 16, 1.45), (3, 17, 16, 1.45), (3, 2, 0, 1.45)):
            with pytest.raises(hs.HairSimError):
                g.tess_stream(abi.TessParams(*bad))
        assert g.tess_stream() == 2 * 3 * 2 * 7 * 2 * 16
        assert g.tess_readback().shape == (2 * 3 * 2 * 7 * 2 * 16, 4)


def test_tess_matches_reference_shader_golden(hs):
    """The GPU pass on the scalp's positions after 60 frames, against the
    reference's own tessellation evaluation shader (tests/golden/ref_tess.npz)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_tess.npz"))
    pos = g["pos"]
    ns = pos.shape[0]
    sim = abi.sim_params_reference(1.45)
    with hs.Context() as ctx:
        gr = ctx.groom_from_state(pos, np.zeros_like(pos), sim)
        for case in ("a", "b"):
            ninst, nlines, nsub, scale = g[f"params_{case}"]
            gr.tess_setup(g[f"faces_{case}"], g["tangents"], g["random"])
            gr.tess_stream(abi.TessParams(int(ninst), int(nlines), int(nsub), float(scale)))
            util.assert_bit_equal(gr.tess_readback(), g[f"out_{case}"], f"tessellation case {case}")
    assert ns == 448
