"""Marschner lookup tables (hs_marschner_luts) on the GPU, against the
oracle's double-precision evaluation of the reference's shaders
(src/shaders/hair/marschner/). The transcendental functions are CUDA's on
the GPU and the C library's on the CPU, so the tables agree to a tolerance
(the float oracle itself is within 1e-6 of the double one for M and 1e-4
for N), and the half tables to the half-precision rounding."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from barbu_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


@pytest.mark.parametrize("res,eta,absorption,ar,br", [(128, 1.55, 0.2, -5.0, 5.0), (64, 1.3, 0.6, -8.0, 3.0)])
def test_tables_match_the_oracle(hs, res, eta, absorption, ar, br):
    torch = pytest.importorskip("torch")
    p = hs.marschner_params_reference()
    p.resolution, p.eta, p.absorption, p.ar, p.br = res, eta, absorption, ar, br
    m64, n64 = oracle.marschner(res, eta, absorption, ar, br, dtype=np.float64)
    with hs.Context() as ctx:
        mf = torch.zeros(res * res * 4, dtype=torch.float32, device="cuda")
        nf = torch.zeros_like(mf)
        mh = torch.zeros(res * res * 4, dtype=torch.float16, device="cuda")
        nh = torch.zeros_like(mh)
        torch.cuda.synchronize()
        ctx.marschner_luts(p, abi.HS_LUT_FLOAT4, mf.data_ptr(), nf.data_ptr())
        ctx.marschner_luts(p, abi.HS_LUT_HALF4, mh.data_ptr(), nh.data_ptr())
        ctx.sync()
        m = mf.cpu().numpy().reshape(res, res, 4).astype(np.float64)
        n = nf.cpu().numpy().reshape(res, res, 4).astype(np.float64)
        mhalf = mh.cpu().numpy().reshape(res, res, 4).astype(np.float64)
        nhalf = nh.cpu().numpy().reshape(res, res, 4).astype(np.float64)
    assert np.isfinite(m).all() and np.isfinite(n).all()
    assert np.abs(m - m64).max() < 2e-6
    dn = np.abs(n - n64)
    assert np.percentile(dn, 99.9) < 1e-5 and dn.max() < 5e-4
    # Half tables: the float tables rounded to half (the reference's RGBA16F).
    np.testing.assert_array_equal(mhalf, m.astype(np.float16).astype(np.float64))
    np.testing.assert_array_equal(nhalf, n.astype(np.float16).astype(np.float64))


def test_table_errors(hs):
    with hs.Context() as ctx:
        p = hs.marschner_params_reference()
        with pytest.raises(hs.HairSimError):
            ctx.marschner_luts(p, abi.HS_LUT_FLOAT4, 0, 0)      # no destination
        p.resolution = 1
        with pytest.raises(hs.HairSimError):
            ctx.marschner_luts(p, abi.HS_LUT_FLOAT4, 16, 0)
        p.resolution = 128
        with pytest.raises(hs.HairSimError):
            ctx.marschner_luts(p, 7, 16, 0)


@pytest.mark.parametrize("k", [0, 1])
def test_tables_match_the_reference_shaders(hs, k):
    """Against the reference's own shaders compiled as C++
    (tests/golden/ref_marschner.npz): CUDA's transcendental functions
    against the C library's, to the float oracle's own distance from
    double (M 2e-6, N 5e-4)."""
    torch = pytest.importorskip("torch")
    from tests import util
    g = util.load_golden("marschner")
    res, eta, absorption, ar, br = (float(x) for x in g[f"params_{k}"])
    res = int(res)
    p = hs.marschner_params_reference()
    p.resolution, p.eta, p.absorption, p.ar, p.br = res, eta, absorption, ar, br
    with hs.Context() as ctx:
        mf = torch.zeros(res * res * 4, dtype=torch.float32, device="cuda")
        nf = torch.zeros_like(mf)
        torch.cuda.synchronize()
        ctx.marschner_luts(p, abi.HS_LUT_FLOAT4, mf.data_ptr(), nf.data_ptr())
        ctx.sync()
        m = mf.cpu().numpy().reshape(res, res, 4)
        n = nf.cpu().numpy().reshape(res, res, 4)
    np.testing.assert_allclose(m, g[f"m_{k}"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(n, g[f"n_{k}"], rtol=0, atol=5e-4)
