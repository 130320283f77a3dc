"""Oracle: the Marschner lookup tables (CPU).

Known answers of the reference's shaders (src/shaders/hair/marschner/):
the M table's w is cos(theta_d), 1 on the diagonal sin(theta_i) =
sin(theta_r); its lobes are Gaussians of the half angle in degrees, so a
lobe peaks where the half angle equals its shift and is symmetric about it;
the N table's w is 1, N_R is the Fresnel term at gamma = -phi/2 (the root
of the p = 0 polynomial, which is linear) over |2 d(phi)/d(gamma)|, and
every entry is in [0, 1]. The float instantiation tracks the double one.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from tests import util


def test_m_table_known_answers():
    res = 128
    m, _ = oracle.marschner(res, dtype=np.float64)
    idx = np.arange(res)
    np.testing.assert_allclose(m[idx, idx, 3], 1.0, atol=1e-12)  # theta_d = 0 on the diagonal
    # R lobe (shift ar = -5 deg, width br = 5): peak value 1 / (sqrt(2 pi) * 5).
    assert abs(m[..., 0].max() - 1.0 / (2.5066282 * 5.0)) < 1e-3
    # Half angle theta_h = (asin(2x/res - 1) + asin(2y/res - 1)) / 2; the R lobe
    # depends on it alone.
    s = 2.0 * idx / res - 1.0
    th = (np.arcsin(s)[None, :] + np.arcsin(s)[:, None]) / 2.0
    deg = th * (180.0 / math.pi)
    want = np.exp(-((deg + 5.0) ** 2) / (2.0 * 25.0)) / (2.5066282 * 5.0)
    np.testing.assert_allclose(m[..., 0], want, rtol=1e-5, atol=1e-9)


def test_n_table_bounds_and_float_tracks_double():
    m32, n32 = oracle.marschner(dtype=np.float32)
    m64, n64 = oracle.marschner(dtype=np.float64)
    assert np.isfinite(n64).all() and (n64 >= 0).all() and (n64 <= 1).all()
    np.testing.assert_array_equal(n64[..., 3], 1.0)
    assert np.abs(m32 - m64).max() < 1e-6
    assert np.abs(n32 - n64).max() < 1e-4


def test_n_r_is_the_fresnel_term_at_minus_half_phi():
    """p = 0: the polynomial is linear, gamma_i = -phi/2 (inc_marschner_n.glsl:40-49)."""
    res = 64
    _, n = oracle.marschner(res, eta=1.55, dtype=np.float64)
    y, x = 48, 20                       # cos(theta_d) = 0.5, cos(phi_d) = -0.375
    ctd = 2.0 * y / res - 1.0
    cpd = 2.0 * x / res - 1.0
    eta = float(np.float32(1.55))         # the table takes eta as a float
    eta_perp = math.sqrt(eta ** 2 - (1 - ctd * ctd)) / ctd
    eta_par = eta ** 2 / eta_perp
    g = -math.acos(cpd) / 2.0

    def ratio(er, na, nb, ci, si):
        st2 = (er * si) ** 2
        if st2 > 1:
            return 1.0
        ct = math.sqrt(1 - st2)
        r = (na * ci - nb * ct) / (na * ci + nb * ct)
        return min(1.0, r * r)

    f = 0.5 * ratio(1 / eta_perp, 1, eta_perp, math.cos(g), math.sin(g)) + \
        0.5 * ratio(1 / eta_par, eta_par, 1, math.cos(g), math.sin(g))
    want = min(f / abs(2.0 * (-2.0) / math.cos(g)), 1.0)
    assert abs(n[y, x, 0] - want) < 1e-12


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_matches_the_reference_marschner_shaders(k):
    """Pinned: the oracle's float tables equal the reference's
    cs_marschner_m.glsl and cs_marschner_n.glsl compiled as C++
    (tests/golden/ref_marschner.npz) bit for bit: the same operations in the
    same order, with the C library's float transcendentals on both sides."""
    g = util.load_golden("marschner")
    res, eta, absorption, ar, br = (float(x) for x in g[f"params_{k}"])
    m, n = oracle.marschner(int(res), eta, absorption, ar, br, dtype=np.float32)
    util.assert_bit_equal(m, g[f"m_{k}"], "M table vs the reference shader")
    util.assert_bit_equal(n, g[f"n_{k}"], "N table vs the reference shader")
    if oracle.ref_marschner_available():
        rm, rn = oracle.ref_marschner(int(res), eta, absorption, ar, br)
        util.assert_bit_equal(rm, g[f"m_{k}"], "reference M rebuilt")
        util.assert_bit_equal(rn, g[f"n_{k}"], "reference N rebuilt")
