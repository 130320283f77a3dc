"""hs_export on the GPU: device-to-device export of positions and
velocities, strand-major (the reference renderer's order,
src/fx/hair.cc:369-392) and point-major, into a caller's device buffer."""
from __future__ import annotations

import numpy as np
import pytest

from barbu_gb300 import abi, scenarios
from tests import util

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


@pytest.mark.parametrize("ns,n", [(1000, 16), (33, 5), (70, 64)])
def test_export_layouts_match_readback(hs, ns, n):
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=ns, npoints=n)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        g.set_spheres(spec.spheres)
        for f in range(3):
            g.set_root_transform(spec.transform((f + 1) / 60))
            g.update(1 / 60)
        pos, vel = g.readback(), g.readback_velocities()
        buf = torch.full((ns * n * 4 + 4,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()  # the fill runs on torch's stream, the export on the context's
        for field, want in ((abi.HS_FIELD_POSITIONS, pos), (abi.HS_FIELD_VELOCITIES, vel)):
            g.export(buf.data_ptr(), buf.numel(), abi.HS_EXPORT_STRAND_MAJOR, field)
            ctx.sync()
            got = buf[: ns * n * 4].cpu().numpy().reshape(ns, n, 4)
            util.assert_bit_equal(got, want, "strand-major export")
            assert np.isnan(buf[-4:].cpu().numpy()).all()  # nothing written past the end
            g.export(buf.data_ptr(), buf.numel(), abi.HS_EXPORT_POINT_MAJOR, field)
            ctx.sync()
            got = buf[: ns * n * 4].cpu().numpy().reshape(n, ns, 4).transpose(1, 0, 2)
            util.assert_bit_equal(got, want, "point-major export")


def test_export_rejects_bad_destinations(hs):
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=64, npoints=8)
    with hs.Context() as ctx:
        g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
        buf = torch.zeros(64 * 8 * 4 + 8, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        with pytest.raises(hs.HairSimError):
            g.export(buf.data_ptr(), 64 * 8 * 4 - 1)          # too small
        with pytest.raises(hs.HairSimError):
            g.export(buf.data_ptr() + 4, buf.numel() - 1)     # misaligned
        host = np.zeros(64 * 8 * 4, np.float32)
        with pytest.raises(hs.HairSimError):
            g.export(host.ctypes.data, host.size)             # host memory
        with pytest.raises(hs.HairSimError):
            g.export(buf.data_ptr(), buf.numel(), layout=7)
