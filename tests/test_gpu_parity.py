"""The CUDA library against the oracle and the golden vectors (GPU).

Every call goes through the C-ABI (libhairsim.so via ctypes). The kernels
follow the same arithmetic contract as the oracle, so in FP32 they must
agree with it bit for bit, in every scene and for every frame. How far FP32
may drift from FP64 is a property of the arithmetic and of the scene's
conditioning, checked on the oracle in tests/test_oracle_dftl.py; here the
FP64 tolerances are checked end to end on the well-conditioned scenes.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu

ONE_STEP_TOL = 1e-5
SEGMENT_TOL = 1e-5
DRIFT_TOL = 1e-3


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


@pytest.fixture(scope="module")
def ctx(hs):
    c = hs.Context()
    yield c
    c.close()


# ---- reference mode: the golden vectors of the reference shader -----------

@pytest.mark.parametrize("case", util.CASES)
def test_reference_mode_bit_exact_with_reference_shader(ctx, case):
    g = util.load_golden(case)
    sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.1, int(g["strand_seed"]))
    sim = abi.sim_params_reference(float(g["scale"]))
    gr = ctx.groom(g["roots"], g["normals"], sp, sim)
    util.assert_bit_equal(gr.readback(), g["pos0"], f"{case} init positions")
    util.assert_bit_equal(gr.readback_velocities(), g["vel0"], f"{case} init velocities")
    p32, v32 = g["pos0"].copy(), g["vel0"].copy()
    for f in range(len(g["dts"])):
        gr.set_bounding_sphere(g["bspheres"][f])
        gr.update(float(g["dts"][f]))
        oracle.frame(p32, v32, sim, float(g["dts"][f]), spheres=g["bspheres"][f][None])
        if f + 1 in g["snap_frames"]:
            k = list(g["snap_frames"]).index(f + 1)
            P, V = gr.readback(), gr.readback_velocities()
            ok = util.finite_strands(g["pos_snap"][k]) & util.finite_strands(g["vel_snap"][k])
            util.assert_bit_equal(P[ok], g["pos_snap"][k][ok], f"{case} frame {f + 1} positions")
            util.assert_bit_equal(V[ok], g["vel_snap"][k][ok], f"{case} frame {f + 1} velocities")
            # The NaN strands of the reference: GPU follows the oracle's guard.
            util.assert_bit_equal(P, p32, f"{case} frame {f + 1} positions vs oracle")
            util.assert_bit_equal(V, v32, f"{case} frame {f + 1} velocities vs oracle")
    gr.destroy()


def test_hair_class_mirrors_reference_update(hs):
    """Hair.init/setup/set_bounding_sphere/update/readback on the scalp."""
    g = util.load_golden("scalp")
    hair = hs.Hair(max_length=0.5, length_scale=float(g["scale"]), seed=int(g["strand_seed"]))
    assert not hair.initialized()
    hair.update(1 / 60)  # uninitialised: a no-op, as in the reference
    hair.init()
    hair.setup(g["roots"], g["normals"])
    assert hair.initialized() and hair.nroots == 448
    for f in range(10):
        hair.set_bounding_sphere(g["bspheres"][f])
        hair.update(float(g["dts"][f]))
    k = list(g["snap_frames"]).index(10)
    util.assert_bit_equal(hair.readback(), g["pos_snap"][k], "Hair after 10 frames")
    hair.deinit()
    assert not hair.initialized()


# ---- DFTL mode: the oracle at small sizes ---------------------------------

def drive(ctx, spec: scenarios.GroomSpec, frames: int, dt: float = 1 / 60, f64: bool = True, gpu_groom=None):
    """Runs spec on the GPU and on the oracle (FP32, and FP64 if asked)."""
    gr = gpu_groom or ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    pos0, vel0 = gr.readback(), gr.readback_velocities()
    p32, v32 = pos0.copy(), vel0.copy()
    p64, v64 = pos0.astype(np.float64), vel0.astype(np.float64)
    rest = pos0[:, 0, :3].copy()
    hist = []
    for f in range(frames):
        t = (f + 1) * dt
        wind = scenarios.wind_at(t) if spec.wind else None
        m = spec.transform(t)
        sph = spec.spheres_at(t)
        if wind is not None:
            gr.set_wind(wind)
        if m is not None:
            gr.set_root_transform(m)
        gr.set_spheres(sph)
        gr.update(dt)
        tg32 = oracle.rigid_targets(rest, m, np.float32) if m is not None else None
        oracle.frame(p32, v32, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=sph, root_targets=tg32)
        if f64:
            tg64 = oracle.rigid_targets(rest, m, np.float64) if m is not None else None
            oracle.frame(p64, v64, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=sph,
                         root_targets=tg64)
        hist.append((gr.readback(), gr.readback_velocities(), p32.copy(), v32.copy(),
                     p64.copy() if f64 else None))
    return gr, pos0, hist


def make_spec(ns, n, substeps=4, iterations=1, nspheres=1, wind=False, roots_mode="none", seed=7, mode="dftl"):
    roots, normals = util.random_roots_on_sphere(ns, seed)
    lengths = np.random.default_rng(seed).uniform(0.3, 0.8, ns).astype(np.float32)
    sp = abi.strand_params(n, abi.HS_LENGTH_TOTAL, 0.5, 0.0, seed)
    root_mode = abi.HS_ROOT_RIGID if roots_mode != "none" else abi.HS_ROOT_PINNED
    if mode == "dftl":
        sim = abi.sim_params_dftl(substeps=substeps, damping=0.9, wind_jitter=0.2 if wind else 0.0,
                                  root_mode=root_mode, iterations=iterations)
    else:
        sim = abi.sim_params_reference(1.45)
        sim.root_mode = root_mode
        sim.substeps = substeps
    spheres = np.zeros((0, 4), np.float32)
    if nspheres == 1:
        spheres = np.array([[0.0, 0.0, 0.0, 1.0]], np.float32)
    elif nspheres > 1:
        spheres = scenarios.shell_spheres(nspheres, seed, d_lo=0.8, d_hi=1.4)
    spec = scenarios.GroomSpec(roots, normals, sp, sim, lengths, spheres, wind=wind)
    if roots_mode == "translate":
        spec.moving_roots, spec.amp = "translate_x", 0.2
    elif roots_mode == "rigid":
        spec.moving_roots, spec.axis, spec.omega_deg, spec.amp, spec.phase = (
            "rigid", np.array([0.0, 0.6, 0.8]), 30.0, 0.3, 0.5)
    return spec


CASES = [
    # (N, substeps, iterations, spheres, wind, roots)
    (2, 1, 1, 1, False, "none"),
    (4, 4, 1, 1, False, "none"),
    (5, 4, 2, 3, True, "translate"),
    (8, 8, 1, 16, True, "rigid"),
    (13, 4, 1, 32, False, "none"),
    (16, 4, 1, 1, False, "translate"),
    (24, 8, 1, 16, True, "rigid"),
    (32, 8, 1, 16, True, "none"),
    (32, 2, 3, 8, True, "rigid"),
    (48, 8, 1, 16, True, "rigid"),
    (40, 3, 1, 8, True, "rigid"),        # odd substep count: a last group of one
    (33, 1, 1, 4, False, "translate"),   # one substep
    (64, 8, 1, 32, True, "none"),
    (64, 2, 2, 4, False, "translate"),
]


@pytest.mark.parametrize("mapping", [abi.HS_MAPPING_THREAD, abi.HS_MAPPING_LANES])
@pytest.mark.parametrize("n,substeps,iterations,nspheres,wind,roots", CASES)
def test_dftl_bit_exact_with_fp32_oracle(ctx, hs, n, substeps, iterations, nspheres, wind, roots, mapping):
    """Both strand mappings: a thread per strand, and a lane group per
    strand (its substeps as a wavefront), where the frame has that form."""
    spec = make_spec(997, n, substeps, iterations, nspheres, wind, roots)
    gr = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    gr.set_mapping(mapping)
    if mapping == abi.HS_MAPPING_LANES and (iterations != 1 or not 2 <= substeps <= 16):
        with pytest.raises(hs.HairSimError) as e:
            gr.update(1 / 60)
        assert e.value.status == abi.HS_ERR_UNSUPPORTED
        gr.destroy()
        return
    assert gr.mapping() == mapping
    gr, pos0, hist = drive(ctx, spec, frames=60, f64=False, gpu_groom=gr)
    for f, (P, V, p32, v32, _) in enumerate(hist):
        util.assert_bit_equal(P, p32, f"frame {f + 1} positions")
        util.assert_bit_equal(V, v32, f"frame {f + 1} velocities")
    gr.destroy()


@pytest.mark.parametrize("n", [8, 16, 32])
def test_dftl_fp64_tolerances_well_conditioned(ctx, n):
    """Hanging strands swinging in the wind, 4 substeps: one-step error <=
    1e-5 x strand length, segment length error <= 1e-5, 60-frame drift <=
    1e-3 x strand length against the FP64 oracle."""
    spec = util.hanging_spec(997, n, substeps=4, spheres=None)
    gr, pos0, hist = drive(ctx, spec, frames=60)
    L = util.strand_lengths(pos0)
    P1, _, p32, _, q1 = hist[0]
    util.assert_bit_equal(P1, p32, "frame 1")
    assert util.max_pos_error_rel(P1, q1, L) <= ONE_STEP_TOL
    s_gpu, s_64 = util.segment_lengths(P1), util.segment_lengths(q1)
    assert np.max(np.abs(s_gpu - s_64) / s_64) <= SEGMENT_TOL
    P60, _, p32, _, q60 = hist[-1]
    util.assert_bit_equal(P60, p32, "frame 60")
    assert util.max_pos_error_rel(P60, q60, L) <= DRIFT_TOL
    gr.destroy()


@pytest.mark.parametrize("n", [8, 16])
def test_dftl_fp64_one_step_with_contacts(ctx, n):
    spec = util.hanging_spec(997, n, substeps=4, spheres="side")
    gr, pos0, hist = drive(ctx, spec, frames=1)
    L = util.strand_lengths(pos0)
    P1, _, p32, _, q1 = hist[0]
    util.assert_bit_equal(P1, p32, "frame 1")
    assert util.max_pos_error_rel(P1, q1, L) <= ONE_STEP_TOL
    gr.destroy()


def test_reference_mode_generalised_to_long_strands(ctx):
    """Reference semantics (gravity x20, 8 iterations, shifted velocity) at N = 16."""
    spec = make_spec(515, 16, substeps=1, nspheres=1, mode="ref")
    gr, pos0, hist = drive(ctx, spec, frames=20, f64=False)
    for f, (P, V, p32, v32, _) in enumerate(hist):
        util.assert_bit_equal(P, p32, f"frame {f + 1} positions")
        util.assert_bit_equal(V, v32, f"frame {f + 1} velocities")
    gr.destroy()


def test_explicit_root_targets(ctx):
    spec = make_spec(300, 8, substeps=4, nspheres=1)
    spec.sim.root_mode = abi.HS_ROOT_EXPLICIT
    gr = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    p32, v32 = gr.readback(), gr.readback_velocities()
    rng = np.random.default_rng(3)
    for f in range(10):
        tg = (p32[:, 0, :3] + rng.normal(scale=0.01, size=(300, 3))).astype(np.float32)
        gr.set_roots(tg)
        gr.set_spheres(spec.spheres)
        gr.update(1 / 60)
        oracle.frame(p32, v32, spec.sim, 1 / 60, seed=7, spheres=spec.spheres, root_targets=tg)
        util.assert_bit_equal(gr.readback(), p32, f"frame {f}")
        np.testing.assert_array_equal(gr.readback()[:, 0, :3], tg)
    gr.destroy()


def test_init_from_state_round_trip(ctx):
    g = util.load_golden("sphere")
    sim = abi.sim_params_reference(float(g["scale"]))
    gr = ctx.groom_from_state(g["pos0"], g["vel0"], sim, seed=int(g["strand_seed"]))
    util.assert_bit_equal(gr.readback(), g["pos0"], "positions")
    util.assert_bit_equal(gr.readback_velocities(), g["vel0"], "velocities")
    gr.set_bounding_sphere(g["bspheres"][0])
    gr.update(float(g["dts"][0]))
    util.assert_bit_equal(gr.readback(), g["pos_snap"][0], "frame 1")
    ptr, lay = gr.device_positions()
    assert ptr and lay.nstrands == 512 and lay.points_per_strand == 4
    assert lay.strand_stride % 32 == 0 and lay.strand_stride >= lay.nstrands
    gr.destroy()


# ---- full size: the large groom (262,144 x 32) ----------------------------

def test_large_groom_full_size_sampled_parity(ctx):
    """All 262,144 strands x 32 points on the GPU for 60 frames; the FP32
    oracle re-runs sampled blocks of strands (strands are independent) and
    must agree bit for bit."""
    spec = scenarios.large()
    gr = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    pos0, vel0 = gr.readback(), gr.readback_velocities()
    rng = np.random.default_rng(11)
    blocks = [(int(b), 256) for b in rng.choice(spec.nstrands - 256, size=8, replace=False)]
    blocks.append((spec.nstrands - 100, 100))  # the last, partial warp
    samp = [(pos0[b:b + k].copy(), vel0[b:b + k].copy()) for b, k in blocks]
    dt = 1 / 60
    for f in range(60):
        t = (f + 1) * dt
        wind = scenarios.wind_at(t)
        gr.set_wind(wind)
        gr.set_spheres(spec.spheres)
        gr.update(dt)
        for (b, k), (p, v) in zip(blocks, samp):
            oracle.frame(p, v, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=spec.spheres, strand_base=b)
        if f in (0, 59):
            P, V = gr.readback(), gr.readback_velocities()
            for (b, k), (p, v) in zip(blocks, samp):
                util.assert_bit_equal(P[b:b + k], p, f"frame {f + 1} strands {b}..{b + k}")
                util.assert_bit_equal(V[b:b + k], v, f"frame {f + 1} strands {b}..{b + k} velocities")
    assert np.isfinite(P).all() and np.isfinite(V).all()
    np.testing.assert_array_equal(util.bits(P[..., 3]), util.bits(pos0[..., 3]))  # rest lengths carried
    gr.destroy()


# ---- errors ---------------------------------------------------------------

def test_invalid_arguments_return_status(ctx, hs):
    roots, normals = util.random_roots_on_sphere(64, 1)
    sim = abi.sim_params_dftl()
    for n in (1, 65):
        with pytest.raises(hs.HairSimError) as e:
            ctx.groom(roots, normals, abi.strand_params(n), sim)
        assert e.value.status == abi.HS_ERR_INVALID_ARG
    bad = roots.copy()
    bad[3, 1] = np.nan
    with pytest.raises(hs.HairSimError) as e:
        ctx.groom(bad, normals, abi.strand_params(8), sim)
    assert e.value.status == abi.HS_ERR_INVALID_ARG
    gr = ctx.groom(roots, normals, abi.strand_params(8), sim)
    with pytest.raises(hs.HairSimError):
        gr.set_spheres(np.zeros((33, 4), np.float32))
    with pytest.raises(hs.HairSimError):
        gr.set_spheres(np.array([[0, 0, 0, -1.0]], np.float32))
    with pytest.raises(hs.HairSimError):
        gr.update(-1.0)
    with pytest.raises(hs.HairSimError):
        gr.update(0.0)  # DFTL divides by the substep
    sim2 = abi.sim_params_dftl(root_mode=abi.HS_ROOT_EXPLICIT)
    gr.set_params(sim2)
    with pytest.raises(hs.HairSimError) as e:
        gr.update(1 / 60)
    assert e.value.status == abi.HS_ERR_NOT_INITIALIZED
    gr.destroy()
