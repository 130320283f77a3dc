"""hs_readback_async / hs_readback_xyz_async / hs_readback_many_async /
hs_readback_wait / hs_readback_drain on the GPU: the copy of frame f runs
on the context's second stream while frame f + 1 updates and is
snapshotted (the staging buffers take turns), into pinned host buffers
that take turns; every frame must equal the blocking hs_readback of a twin
groom (the xyz forms its first three components), and the ordering against
the blocking readbacks (which share the first staging buffer) must hold."""
from __future__ import annotations

import numpy as np
import pytest

from tests import util
from barbu_gb300 import scenarios

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hs(built_library):
    from barbu_gb300 import hairsim
    return hairsim


def _pinned(torch, ns, n):
    t = torch.empty((ns, n, 4), dtype=torch.float32, pin_memory=True)
    t.fill_(float("nan"))
    return t.numpy()


def _groom(ctx, spec):
    g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
    g.set_spheres(spec.spheres)
    return g


def _step(g, spec, f):
    g.set_root_transform(spec.transform((f + 1) / 60))
    g.update(1 / 60)


@pytest.mark.parametrize("ns,n", [(1000, 16), (70, 64)])
def test_pipelined_frames_match_blocking_readback(hs, ns, n):
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=ns, npoints=n)
    frames = 6
    with hs.Context() as ctx:
        twin = _groom(ctx, spec)
        want = []
        for f in range(frames):
            _step(twin, spec, f)
            want.append(twin.readback())
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        bufs = [_pinned(torch, ns, n), _pinned(torch, ns, n)]
        got = []
        for f in range(frames):
            _step(g, spec, f)
            if f:
                ctx.readback_wait()
                got.append(bufs[(f - 1) % 2].copy())
            g.readback_async(bufs[f % 2])
        ctx.readback_wait()
        got.append(bufs[(frames - 1) % 2].copy())
    for f in range(frames):
        util.assert_bit_equal(got[f], want[f], f"frame {f} positions")


def test_many_grooms_one_wait(hs):
    torch = pytest.importorskip("torch")
    specs = [scenarios.plain(ns=ns, npoints=n) for ns, n in ((257, 8), (64, 32), (1000, 12))]
    with hs.Context() as ctx:
        grooms = [_groom(ctx, s) for s in specs]
        for f in range(3):
            for g, s in zip(grooms, specs):
                _step(g, s, f)
        want = [g.readback() for g in grooms]
        bufs = [_pinned(torch, s.nstrands, s.npoints) for s in specs]
        for g, b in zip(grooms, bufs):
            g.readback_async(b)
        ctx.readback_wait()
        for w, b in zip(want, bufs):
            util.assert_bit_equal(b, w, "positions")


def test_blocking_readback_after_async_keeps_order(hs):
    """The velocity readback reuses the staging buffer the asynchronous
    position copy reads: it must wait for that copy on the device."""
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=4096, npoints=32)
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        for f in range(2):
            _step(g, spec, f)
        pos, vel = g.readback(), g.readback_velocities()
        buf = _pinned(torch, spec.nstrands, spec.npoints)
        for _ in range(3):
            g.readback_async(buf)
            got_vel = g.readback_velocities()
            ctx.readback_wait()
            util.assert_bit_equal(buf, pos, "positions (asynchronous)")
            util.assert_bit_equal(got_vel, vel, "velocities (blocking)")


def test_destroy_with_copy_in_flight(hs):
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=4096, npoints=32)
    buf = _pinned(torch, spec.nstrands, spec.npoints)
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        _step(g, spec, 0)
        want = g.readback()
        g.readback_async(buf)
        g.destroy()  # waits for the copy before freeing the staging buffer
        ctx.readback_wait()
    util.assert_bit_equal(buf, want, "positions")


def test_async_rejects_small_buffer(hs):
    spec = scenarios.plain(ns=64, npoints=8)
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        small = np.zeros((64, 8, 4), np.float32)[:, :7]
        with pytest.raises(ValueError):
            g.readback_async(small)  # not contiguous
        with pytest.raises(hs.HairSimError):
            g.readback_async(np.zeros(64 * 8 * 4 - 1, np.float32))
        ctx.readback_wait()  # nothing queued: returns at once


@pytest.mark.parametrize("ns,n", [(1000, 16), (33, 5), (70, 64)])
def test_xyz_readbacks_match_xyzw(hs, ns, n):
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=ns, npoints=n)
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        t = [torch.empty((ns, n, 3), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        bufs = [x.numpy() for x in t]
        for f in range(4):
            _step(g, spec, f)
            want = g.readback()
            util.assert_bit_equal(g.readback_xyz(), np.ascontiguousarray(want[..., :3]), f"frame {f} xyz")
            g.readback_xyz_async(bufs[f % 2])
            ctx.readback_wait()
            util.assert_bit_equal(bufs[f % 2], np.ascontiguousarray(want[..., :3]), f"frame {f} xyz (asynchronous)")
        with pytest.raises(hs.HairSimError):
            g.readback_xyz(np.zeros(ns * n * 3 - 1, np.float32))


def _want_frames(hs, specs, frames):
    with hs.Context() as ctx:
        twins = [_groom(ctx, s) for s in specs]
        want = []
        for f in range(frames):
            for g, s in zip(twins, specs):
                _step(g, s, f)
            want.append([g.readback() for g in twins])
    return want


@pytest.mark.parametrize("comps", [3, 4])
def test_two_in_flight_with_drain(hs, comps):
    """Frame f + 1's readback is queued before frame f's is waited for
    (drain to 1): each groom's two staging buffers and the two host buffers
    take turns, and every frame arrives whole."""
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=1500, npoints=24)
    frames = 7
    want = _want_frames(hs, [spec], frames)
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        bufs = [torch.empty((spec.nstrands, spec.npoints, comps), dtype=torch.float32, pin_memory=True).numpy()
                for _ in range(2)]
        got = []
        for f in range(frames):
            _step(g, spec, f)
            (g.readback_xyz_async if comps == 3 else g.readback_async)(bufs[f % 2])
            ctx.readback_drain(1)
            if f:
                got.append(bufs[(f - 1) % 2].copy())
        ctx.readback_drain(0)
        got.append(bufs[(frames - 1) % 2].copy())
    for f in range(frames):
        util.assert_bit_equal(got[f], np.ascontiguousarray(want[f][0][..., :comps]), f"frame {f}")


@pytest.mark.parametrize("comps", [3, 4])
def test_many_async_matches_blocking_readbacks(hs, comps):
    """hs_readback_many_async: every groom's strand-major frame in list
    order in one host buffer, pipelined two frames deep like the bench."""
    torch = pytest.importorskip("torch")
    specs = [scenarios.plain(ns=ns, npoints=n) for ns, n in ((257, 8), (64, 32), (1000, 12), (33, 5))]
    frames = 5
    want = _want_frames(hs, specs, frames)
    total = sum(s.nstrands * s.npoints * comps for s in specs)
    with hs.Context() as ctx:
        grooms = [_groom(ctx, s) for s in specs]
        handles = ctx.handles_of(grooms)
        bufs = [torch.empty(total, dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
        got = []
        for f in range(frames):
            for g, s in zip(grooms, specs):
                _step(g, s, f)
            ctx.readback_many_async(grooms, bufs[f % 2], comps=comps, handles=handles)
            ctx.readback_drain(1)
            if f:
                got.append(bufs[(f - 1) % 2].copy())
        ctx.readback_wait()
        got.append(bufs[(frames - 1) % 2].copy())
        with pytest.raises(hs.HairSimError):
            ctx.readback_many_async(grooms, np.zeros(total - 1, np.float32), comps=comps)
        with pytest.raises(hs.HairSimError):
            ctx.readback_many_async(grooms, np.zeros(total, np.float32), comps=2)
    for f in range(frames):
        at = 0
        for k, s in enumerate(specs):
            size = s.nstrands * s.npoints * comps
            part = got[f][at:at + size].reshape(s.nstrands, s.npoints, comps)
            util.assert_bit_equal(part, np.ascontiguousarray(want[f][k][..., :comps]), f"frame {f} groom {k}")
            at += size


def test_third_readback_waits_for_the_first(hs):
    """Three readbacks of one groom in flight: the third reuses the first's
    staging buffer and must wait on the device for its copy."""
    torch = pytest.importorskip("torch")
    spec = scenarios.plain(ns=4096, npoints=32)
    want = _want_frames(hs, [spec], 3)
    with hs.Context() as ctx:
        g = _groom(ctx, spec)
        bufs = [_pinned(torch, spec.nstrands, spec.npoints) for _ in range(3)]
        for f in range(3):
            _step(g, spec, f)
            g.readback_async(bufs[f])
        ctx.readback_drain(0)
    for f in range(3):
        util.assert_bit_equal(bufs[f], want[f][0], f"frame {f}")


def test_many_async_rejects_a_foreign_groom(hs):
    spec = scenarios.plain(ns=64, npoints=8)
    with hs.Context() as a, hs.Context() as b:
        ga, gb = _groom(a, spec), _groom(b, spec)
        with pytest.raises(hs.HairSimError):
            a.readback_many_async([ga, gb], np.zeros(2 * 64 * 8 * 3, np.float32))
        a.readback_drain(0)  # nothing queued
