"""Per-groom frame statistics (hs_groom_stats) on the GPU: bounds, kinetic
energy and largest speed, reduced inside the step kernel with warp shuffles
per 32-strand tile. Bounds are exact; the energy is a float sum in a fixed
order (per strand in point order, then a shuffle tree, then the tiles in
double), so it matches a double sum of the same velocities to ~1e-6."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import scenarios

pytestmark = pytest.mark.gpu

DT = 1 / 60


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def expected(pos, vel):
    p = pos[..., :3].reshape(-1, 3).astype(np.float64)
    v = vel[..., :3].reshape(-1, 3).astype(np.float64)
    v2 = (v * v).sum(axis=1)
    return p.min(axis=0), p.max(axis=0), 0.5 * v2.sum(), np.sqrt(v2.max())


@pytest.mark.parametrize("ns,n", [(4096, 16), (300, 8), (1000, 32), (77, 64)])
def test_stats_match_the_state(hs, ns, n):
    spec = scenarios.plain(ns=ns, npoints=n)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        b = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        assert g.stats() is None
        for f in range(4):
            m = spec.transform((f + 1) * DT)
            for x in (g, b):
                x.set_root_transform(m)
                x.set_spheres(spec.spheres_at((f + 1) * DT))
            g.update(DT)
            ctx.update_many([b], DT)
        st, sb = g.stats(), b.stats()
        pos, vel = g.readback(), g.readback_velocities()
    lo, hi, ke, vmax = expected(pos, vel)
    np.testing.assert_array_equal(np.asarray(st["bounds_min"], np.float64), lo)
    np.testing.assert_array_equal(np.asarray(st["bounds_max"], np.float64), hi)
    assert abs(st["kinetic_energy"] - ke) <= 1e-5 * ke + 1e-12
    assert abs(st["max_speed"] - vmax) <= 1e-6 * vmax + 1e-12
    assert st == sb  # the batched kernels reduce the same tiles the same way


def test_stats_of_reference_mode_and_after_autotune(hs):
    g0 = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "ref_scalp.npz"))
    from barbu_gb300 import abi
    sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.1, int(g0["strand_seed"]))
    with hs.Context() as ctx:
        g = ctx.groom(g0["roots"], g0["normals"], sp, abi.sim_params_reference(float(g0["scale"])))
        g.set_bounding_sphere(g0["bspheres"][0])
        g.update(float(g0["dts"][0]))
        st = g.stats()
        pos, vel = g.readback(), g.readback_velocities()
        lo, hi, ke, vmax = expected(pos, vel)
        np.testing.assert_array_equal(np.asarray(st["bounds_min"], np.float64), lo)
        assert abs(st["kinetic_energy"] - ke) <= 1e-5 * ke + 1e-12
        ctx.autotune([g], float(g0["dts"][1]))
        assert g.stats() is None  # the trial frames were undone
    # and the GPU state is the oracle's (the stats describe the real frame)
    p, v = oracle.init(g0["roots"], g0["normals"], sp, dtype=np.float32)
    oracle.frame(p, v, abi.sim_params_reference(float(g0["scale"])), float(g0["dts"][0]),
                 seed=int(sp.seed), spheres=g0["bspheres"][0][None])
    np.testing.assert_array_equal(p.view(np.uint32), pos.view(np.uint32))
