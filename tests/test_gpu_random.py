"""Randomised shapes across every kernel form (GPU).

Each case draws a groom shape (points, substeps, iterations, spheres, root
motion, wind, strand count, arithmetic contract) and runs it through a
thread per strand, a lane group per strand (where the frame has that form),
the batched update and the batched update without allocation. All forms
must give the same bits; under the EXACT contract they must also equal the
FP32 oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu

DT = 1 / 60
FRAMES = 4


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def draw(seed):
    rng = np.random.default_rng(1000 + seed)
    ns = int(rng.integers(1, 700))
    n = int(rng.integers(2, 65))
    substeps = int(rng.choice([1, 2, 3, 4, 5, 8, 12, 16]))
    iterations = int(rng.choice([1, 1, 1, 2]))
    nspheres = int(rng.integers(0, 33))
    rigid = bool(rng.integers(0, 2))
    contract = int(rng.choice([abi.HS_CONTRACT_EXACT, abi.HS_CONTRACT_FAST]))
    roots, normals = util.random_roots_on_sphere(ns, seed)
    lengths = rng.uniform(0.2, 0.9, ns).astype(np.float32)
    sp = abi.strand_params(n, abi.HS_LENGTH_TOTAL, 0.5, 0.0, seed)
    sim = abi.sim_params_dftl(substeps=substeps, damping=float(rng.uniform(0.5, 1.0)),
                              wind_jitter=float(rng.uniform(0.0, 0.3)),
                              root_mode=abi.HS_ROOT_RIGID if rigid else abi.HS_ROOT_PINNED,
                              iterations=iterations, contract=contract)
    spheres = scenarios.shell_spheres(nspheres, seed, d_lo=0.7, d_hi=1.5) if nspheres else \
        np.zeros((0, 4), np.float32)
    spec = scenarios.GroomSpec(roots, normals, sp, sim, lengths, spheres, wind=True)
    if rigid:
        spec.moving_roots, spec.axis, spec.omega_deg, spec.amp, spec.phase = (
            "rigid", np.array([0.3, 0.8, 0.5]), float(rng.uniform(0, 40)), 0.3, float(rng.uniform(0, 6)))
    return spec


def feed(g, spec, f):
    t = (f + 1) * DT
    m = spec.transform(t)
    if m is not None:
        g.set_root_transform(m)
    g.set_wind(scenarios.wind_at(t))
    g.set_spheres(spec.spheres_at(t))


@pytest.mark.parametrize("seed", range(16))
def test_random_shape_same_bits_in_every_form(hs, seed):
    spec = draw(seed)
    sim = spec.sim
    lanes_ok = sim.iterations == 1 and 2 <= sim.substeps <= 16
    with hs.Context() as ctx:
        make = lambda: ctx.groom(spec.roots, spec.normals, spec.strand, sim, lengths=spec.lengths)  # noqa: E731
        thread, lanes, batched, noalloc = make(), make(), make(), make()
        thread.set_mapping(abi.HS_MAPPING_THREAD)
        lanes.set_mapping(abi.HS_MAPPING_LANES if lanes_ok else abi.HS_MAPPING_THREAD)
        pos0, vel0 = thread.readback(), thread.readback_velocities()
        for f in range(FRAMES):
            for g in (thread, lanes, batched, noalloc):
                feed(g, spec, f)
            thread.update(DT)
            lanes.update(DT)
            ctx.update_many([batched], DT)
            ctx.update_many_noalloc([noalloc], DT)
        want_p, want_v = thread.readback(), thread.readback_velocities()
        for g, what in ((lanes, "lane groups"), (batched, "batched"), (noalloc, "no-alloc batched")):
            util.assert_bit_equal(g.readback(), want_p, f"seed {seed}: {what} positions")
            util.assert_bit_equal(g.readback_velocities(), want_v, f"seed {seed}: {what} velocities")
        for g in (thread, lanes, batched, noalloc):
            g.destroy()
    if sim.contract == abi.HS_CONTRACT_EXACT:
        p, v = pos0.copy(), vel0.copy()
        rest = pos0[:, 0, :3].copy()
        for f in range(FRAMES):
            t = (f + 1) * DT
            m = spec.transform(t)
            tg = oracle.rigid_targets(rest, m, np.float32) if m is not None else None
            oracle.frame(p, v, sim, DT, seed=int(spec.strand.seed), wind=scenarios.wind_at(t),
                         spheres=spec.spheres_at(t), root_targets=tg)
        util.assert_bit_equal(want_p, p, f"seed {seed}: positions vs the FP32 oracle")
        util.assert_bit_equal(want_v[..., :3], v[..., :3], f"seed {seed}: velocities vs the FP32 oracle")
