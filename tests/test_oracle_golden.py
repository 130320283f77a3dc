"""The oracle against the golden vectors of the reference shader (CPU).

The golden vectors are the output of src/shaders/hair/01_simulation/
cs_simulation.glsl itself, compiled as C++ (tests/golden/make_golden.py).
These tests pin the oracle before anything is compared against it.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import abi
from tests import util


def run_oracle(g, dtype):
    sim = abi.sim_params_reference(float(g["scale"]))
    p = g["pos0"].astype(dtype)
    v = g["vel0"].astype(dtype)
    snaps = {}
    for f in range(len(g["dts"])):
        oracle.frame(p, v, sim, float(g["dts"][f]), spheres=g["bspheres"][f][None])
        if f + 1 in g["snap_frames"]:
            snaps[f + 1] = (p.copy(), v.copy())
    return snaps


@pytest.mark.parametrize("case", util.CASES)
def test_oracle_fp32_is_bit_exact_with_reference_shader(case):
    g = util.load_golden(case)
    snaps = run_oracle(g, np.float32)
    for k, f in enumerate(g["snap_frames"]):
        ref_p, ref_v = g["pos_snap"][k], g["vel_snap"][k]
        ok = util.finite_strands(ref_p) & util.finite_strands(ref_v)
        p, v = snaps[int(f)]
        util.assert_bit_equal(p[ok], ref_p[ok], f"{case} frame {f} positions")
        util.assert_bit_equal(v[ok], ref_v[ok], f"{case} frame {f} velocities")
        # Where the reference produced NaN (two coincident control points,
        # normalize(0)), the oracle's documented guard stays finite.
        assert np.isfinite(p[~ok]).all() and np.isfinite(v[~ok]).all()


def test_edge_fixture_contains_the_reference_nan_case():
    g = util.load_golden("edge")
    assert not util.finite_strands(g["pos_snap"][-1]).all(), "edge case should show the reference's NaN"


@pytest.mark.parametrize("case", ("scalp", "sphere"))
def test_oracle_fp64_within_tolerance_of_reference_shader(case):
    """FP32 reference vs FP64 restatement: one-step max position error
    <= 1e-5 x strand length; 60-frame drift <= 1e-3 x strand length."""
    g = util.load_golden(case)
    snaps = run_oracle(g, np.float64)
    L = util.strand_lengths(g["pos0"], float(g["scale"]))
    frames = list(g["snap_frames"])
    one = frames.index(1)
    err1 = util.max_pos_error_rel(g["pos_snap"][one], snaps[1][0], L)
    assert err1 <= 1e-5, err1
    last = frames.index(60)
    err60 = util.max_pos_error_rel(g["pos_snap"][last], snaps[60][0], L)
    assert err60 <= 1e-3, err60


def test_oracle_init_reproduces_fixture_state():
    for case in util.CASES:
        g = util.load_golden(case)
        sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.1, int(g["strand_seed"]))
        p, v = oracle.init(g["roots"], g["normals"], sp, dtype=np.float32)
        util.assert_bit_equal(p, g["pos0"], f"{case} init positions")
        util.assert_bit_equal(v, g["vel0"], f"{case} init velocities")


def test_reference_init_layout_rule():
    """Hair::init_simulation: offset_i = i*(maxlength/N)*rv, w_i = offset_i -
    offset_{i-1}, root w = 0, velocity 0 (src/fx/hair.cc:262-288)."""
    roots = np.array([[0.0, 0.0, 0.0], [1.0, 2.0, 3.0]], np.float32)
    normals = np.array([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0]], np.float32)
    sp = abi.strand_params(4, abi.HS_LENGTH_REFERENCE, 0.5, 0.0, 0)
    p, v = oracle.init(roots, normals, sp, dtype=np.float64)
    np.testing.assert_allclose(p[0, :, 1], [0.0, 0.125, 0.25, 0.375])
    np.testing.assert_allclose(p[0, :, 3], [0.0, 0.125, 0.125, 0.125])
    np.testing.assert_allclose(p[1, :, 0], [1.0, 1.125, 1.25, 1.375])
    assert not v.any()


@pytest.mark.skipif(not oracle.ref_glsl_available(), reason="reference tree not present here")
@pytest.mark.parametrize("case", util.CASES)
def test_reference_shader_reproduces_its_fixtures(case):
    """The committed fixtures are what the reference shader computes."""
    g = util.load_golden(case)
    p, v = g["pos0"].copy(), g["vel0"].copy()
    for f in range(len(g["dts"])):
        p, v = oracle.ref_glsl_frame(p, v, float(g["dts"][f]), float(g["scale"]), g["bspheres"][f])
        if f + 1 in g["snap_frames"]:
            k = list(g["snap_frames"]).index(f + 1)
            np.testing.assert_array_equal(util.bits(p), util.bits(g["pos_snap"][k]))
            np.testing.assert_array_equal(util.bits(v), util.bits(g["vel_snap"][k]))


def test_golden_cases_exercise_collisions():
    for case in ("scalp", "sphere"):
        g = util.load_golden(case)
        p = g["pos_snap"][-1][..., :3]
        bs = g["bspheres"][g["snap_frames"][-1] - 1]
        on = np.abs(np.linalg.norm(p - bs[:3], axis=-1) - bs[3]) < 1e-5
        assert on[:, 1:].sum() > 100, case


def test_golden_pin_catches_a_one_ulp_change():
    """Bit equality with the golden vectors is a sharp check: the FP32
    oracle with the first frame's time step moved by one ulp no longer
    matches them."""
    g = {k: np.array(v) for k, v in util.load_golden("sphere").items()}
    g["dts"] = g["dts"].astype(np.float32)
    g["dts"][0] = np.nextafter(g["dts"][0], np.float32(1))
    snaps = run_oracle(g, np.float32)
    f = int(g["snap_frames"][0])
    ok = util.finite_strands(g["pos_snap"][0])
    with pytest.raises(AssertionError):
        util.assert_bit_equal(snaps[f][0][ok], g["pos_snap"][0][ok], "positions")
