"""Lane groups (GPU): a group of K lanes per strand, lane k running substep
k as a wavefront (hs_mapping LANES, hs_variant LANES).

The frames must be bit-identical to the thread-per-strand kernels' and to
the FP32 oracle: the arithmetic of every point and substep is the same,
only which lane does it changes. The DFTL parity cases of test_gpu_parity
run under both mappings; these add the skinned groom (many spheres, the
register-cached push), the widest groups, the statistics, the AUTO choice,
and the batched variant pinned or chosen by the autotuner.
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


def test_auto_mapping_takes_lanes_for_small_grooms_only(hs):
    with hs.Context() as ctx:
        small = scenarios.plain(ns=4096, npoints=16)  # 128 tiles: lanes
        g = ctx.groom(small.roots, small.normals, small.strand, small.sim)
        assert g.mapping() == abi.HS_MAPPING_LANES
        g.set_mapping(abi.HS_MAPPING_THREAD)
        assert g.mapping() == abi.HS_MAPPING_THREAD
        g.set_mapping(abi.HS_MAPPING_AUTO)
        # One substep, or several iterations: no lane-group form.
        for sub, it in ((1, 1), (4, 2)):
            g.set_params(abi.sim_params_dftl(substeps=sub, iterations=it, root_mode=abi.HS_ROOT_RIGID))
            assert g.mapping() == abi.HS_MAPPING_THREAD
        g.destroy()
        big = scenarios.plain(ns=131072, npoints=16)  # 4,096 tiles: a thread per strand fills the GPU
        g = ctx.groom(big.roots, big.normals, big.strand, big.sim)
        assert g.mapping() == abi.HS_MAPPING_THREAD
        with pytest.raises(hs.HairSimError):
            g.set_mapping(3)
        g.destroy()


def test_lanes_rejected_where_the_frame_has_no_lane_form(hs):
    spec = scenarios.plain(ns=64, npoints=8)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        g.set_mapping(abi.HS_MAPPING_LANES)
        for sim in (abi.sim_params_dftl(substeps=1), abi.sim_params_dftl(substeps=17),
                    abi.sim_params_dftl(substeps=4, iterations=2), abi.sim_params_reference(1.45)):
            g.set_params(sim)
            with pytest.raises(hs.HairSimError) as e:
                g.update(DT)
            assert e.value.status == abi.HS_ERR_UNSUPPORTED
        g.destroy()


@pytest.mark.parametrize("ns,n,nsph,substeps", [(700, 64, 32, 8), (300, 16, 8, 16), (97, 8, 0, 2)])
def test_skinned_lanes_bit_exact_vs_oracle(hs, ns, n, nsph, substeps):
    spec = scenarios.skinned(ns=ns, npoints=n, nspheres=nsph, substeps=substeps)
    sp = spec.strand
    p, v = oracle.init(spec.roots, spec.normals, sp, dtype=np.float32)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
        g.set_skin(spec.bones, spec.weights)
        g.set_mapping(abi.HS_MAPPING_LANES)
        for f in range(10):
            m = spec.rig.matrices(f + 1)
            g.set_bone_matrices(m)
            g.set_spheres(spec.spheres_at(f + 1))
            g.update(DT)
            tg = oracle.skin_targets(spec.roots, spec.bones, spec.weights, oracle.matrix_to_dual_quat(m),
                                     dtype=np.float32)
            oracle.frame(p, v, spec.sim, DT, seed=int(sp.seed), spheres=spec.spheres_at(f + 1), root_targets=tg)
        util.assert_bit_equal(g.readback(), p, "positions")
        util.assert_bit_equal(g.readback_velocities()[..., :3], v[..., :3], "velocities")
        g.destroy()


def test_lanes_statistics_match_thread_per_strand(hs):
    spec = scenarios.plain(ns=1000, npoints=24)
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        b = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        a.set_mapping(abi.HS_MAPPING_THREAD)
        b.set_mapping(abi.HS_MAPPING_LANES)
        for f in range(5):
            for g in (a, b):
                g.set_root_transform(spec.transform((f + 1) * DT))
                g.set_spheres(spec.spheres_at((f + 1) * DT))
                g.update(DT)
            sa, sb = a.stats(), b.stats()
            assert sa.keys() == sb.keys()
            for key in sa:
                assert np.array_equal(np.asarray(sa[key]), np.asarray(sb[key])), (f, key, sa[key], sb[key])
        util.assert_bit_equal(b.readback(), a.readback(), "positions")
        a.destroy()
        b.destroy()


def batch_specs():
    specs = scenarios.batched(ngrooms=6, scale=0.02)  # DFTL, S = 8, N in {8..32}
    specs.append(scenarios.plain(ns=333, npoints=12))  # S = 4
    return specs


def run_batched(hs, specs, pin=None, frames=8):
    with hs.Context() as ctx:
        if pin is not None:
            for pts in (8, 16, 24, 32):
                ctx.tune_override(pts, abi.HS_MODE_DFTL, abi.HS_VARIANT_LANES, pin, 1)
        gs = [ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths) for s in specs]
        for f in range(frames):
            t = (f + 1) * DT
            for g, s in zip(gs, specs):
                m = s.transform(t)
                if m is not None:
                    g.set_root_transform(m)
                if s.wind:
                    g.set_wind(scenarios.wind_at(t))
                g.set_spheres(s.spheres_at(t))
            ctx.update_many(gs, DT)
        out = [(g.readback(), g.readback_velocities()) for g in gs]
        for g in gs:
            g.destroy()
    return out


@pytest.mark.parametrize("pin", [8, 16, 2])
def test_batched_lanes_bit_identical(hs, pin):
    """Pinned lane groups of 8 and 16 run the batch; groups of 2 are too
    narrow for its 8-substep grooms, which then take the default shape."""
    specs = batch_specs()
    want = run_batched(hs, specs)
    got = run_batched(hs, specs, pin=pin)
    for k, ((p, v), (pw, vw)) in enumerate(zip(got, want)):
        util.assert_bit_equal(p, pw, f"groom {k} positions")
        util.assert_bit_equal(v, vw, f"groom {k} velocities")


def test_autotuner_searches_lane_groups(hs):
    """A small groom alone in a batch: the tuner times lane groups among
    its shapes; the chosen shape is reported and runs bit-identically."""
    spec = scenarios.plain(ns=4096, npoints=16)
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        b = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        b.set_mapping(abi.HS_MAPPING_THREAD)
        trials = ctx.autotune([a], DT)
        assert trials > 0
        entries = ctx.tune_entries()
        assert len(entries) == 1
        for f in range(4):
            for g in (a, b):
                g.set_root_transform(spec.transform((f + 1) * DT))
                g.set_spheres(spec.spheres_at((f + 1) * DT))
            ctx.update_many([a], DT)
            b.update(DT)
        util.assert_bit_equal(a.readback(), b.readback(), "positions")
        a.destroy()
        b.destroy()


@pytest.mark.parametrize("n,substeps", [(2, 4), (3, 2), (5, 16)])
def test_lanes_shortest_strands_match_thread_per_strand(hs, n, substeps):
    """The wavefront's head and tail overlap when a strand has 2 or 3
    points: every step is both, and the frames still match."""
    spec = scenarios.plain(ns=300, npoints=n)
    sim = abi.sim_params_dftl(substeps=substeps, damping=0.9, wind_jitter=0.2, root_mode=abi.HS_ROOT_RIGID)
    with hs.Context() as ctx:
        a = ctx.groom(spec.roots, spec.normals, spec.strand, sim)
        b = ctx.groom(spec.roots, spec.normals, spec.strand, sim)
        a.set_mapping(abi.HS_MAPPING_THREAD)
        b.set_mapping(abi.HS_MAPPING_LANES)
        for f in range(8):
            t = (f + 1) * DT
            for g in (a, b):
                g.set_root_transform(spec.transform(t))
                g.set_spheres(spec.spheres_at(t))
                g.set_wind(scenarios.wind_at(t))
                g.update(DT)
        util.assert_bit_equal(b.readback(), a.readback(), "positions")
        util.assert_bit_equal(b.readback_velocities(), a.readback_velocities(), "velocities")
        a.destroy()
        b.destroy()
