"""Served stream (hs_server_*) on the GPU.

Continuous batching: requests arrive while others are on the GPU, are
admitted as slots and memory free up, and all resident grooms advance in
one launch per tick. Each result must be the same alone and in the mix
(bit for bit: a groom's frames depend only on its own state, inputs and
elapsed time), the budget must never be exceeded, and admission must follow
arrival order.
"""
from __future__ import annotations

import math

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


def request_spec(ns, n, seed, nspheres=4, substeps=4):
    roots, normals = scenarios.icosphere_roots(ns, seed, subdiv=3)
    lengths = np.random.default_rng(seed).uniform(0.3, 0.8, ns).astype(np.float32)
    sp = abi.strand_params(n, abi.HS_LENGTH_TOTAL, 0.5, 0.0, seed)
    sim = abi.sim_params_dftl(substeps=substeps, damping=0.9, wind_jitter=0.2)
    spheres = scenarios.shell_spheres(nspheres, seed)
    return dict(roots=roots, normals=normals, strand=sp, sim=sim, spheres=spheres, lengths=lengths,
                wind=(0.0, 0.0, 0.5), swing_amp=1.5, swing_omega=0.7)


def submit(srv, spec, frames, keep=False):
    return srv.submit(spec["roots"], spec["normals"], spec["strand"], spec["sim"], frames, spheres=spec["spheres"],
                      wind=spec["wind"], swing_amp=spec["swing_amp"], swing_omega=spec["swing_omega"], keep=keep,
                      lengths=spec["lengths"])


def run_until_done(srv, tickets, max_ticks=2000):
    for _ in range(max_ticks):
        if all(srv.poll(t)[0] in (abi.HS_REQ_DONE, abi.HS_REQ_GONE) for t in tickets):
            return
        srv.tick(DT)
    raise AssertionError("requests did not finish")


def test_result_same_alone_and_in_the_mix(hs):
    target = request_spec(3000, 32, 101)
    frames = 25
    with hs.Context() as ctx:
        with hs.Server(ctx, budget_bytes=1 << 30) as srv:
            t = submit(srv, target, frames, keep=True)
            run_until_done(srv, [t])
            alone_p, alone_v = srv.collect(t)
        with hs.Server(ctx, budget_bytes=1 << 30) as srv:
            others = [request_spec(500 + 700 * k, [8, 16, 24, 32, 48][k % 5], 200 + k) for k in range(6)]
            tickets = [submit(srv, others[0], 40), submit(srv, others[1], 7)]
            for _ in range(3):
                srv.tick(DT)
            t = submit(srv, target, frames, keep=True)  # arrives while others run
            for k in range(2, 6):
                srv.tick(DT)
                tickets.append(submit(srv, others[k], 10 + 5 * k))
            run_until_done(srv, tickets + [t])
            mix_p, mix_v = srv.collect(t)
    util.assert_bit_equal(mix_p, alone_p, "positions alone vs mix")
    util.assert_bit_equal(mix_v, alone_v, "velocities alone vs mix")
    # And both match the oracle running the same request frame by frame.
    sp = target["strand"]
    p, v = oracle.init(target["roots"], target["normals"], sp, dtype=np.float32, lengths=target["lengths"])
    dt32 = float(np.float32(DT))
    amp, om = float(np.float32(1.5)), float(np.float32(0.7))
    for f in range(frames):
        # The server's wind: wind + (float)(amp * sin(omega * t)), t = (frames done + 1) * dt, in double.
        t = (f + 1) * dt32
        w = np.array([np.float32(0.0) + np.float32(amp * math.sin(om * t)), 0.0, 0.5], np.float32)
        oracle.frame(p, v, target["sim"], DT, seed=int(sp.seed), wind=w, spheres=target["spheres"])
    util.assert_bit_equal(alone_p, p, "served positions vs oracle")


def test_budget_fifo_admission_and_retirement(hs):
    specs = [request_spec(2000 + 1000 * (k % 4), 16, 300 + k, nspheres=2) for k in range(10)]
    sizes = [abi.groom_state_bytes(s["roots"].shape[0], 16) for s in specs]
    budget = 3 * max(sizes) + 4096
    with hs.Context() as ctx, hs.Server(ctx, budget_bytes=budget) as srv:
        frames = [5 + (k % 3) * 4 for k in range(10)]
        tickets = [submit(srv, s, f) for s, f in zip(specs, frames)]
        admitted_order = []
        seen = set()
        for _ in range(400):
            st = srv.tick(DT)
            assert st.resident_bytes <= budget
            for k, t in enumerate(tickets):
                state, _ = srv.poll(t)
                if state != abi.HS_REQ_QUEUED and t not in seen:
                    seen.add(t)
                    admitted_order.append(k)
            if all(srv.poll(t)[0] == abi.HS_REQ_GONE for t in tickets):
                break
        assert admitted_order == sorted(admitted_order), admitted_order  # first come, first served
        assert len(seen) == len(tickets)
        assert all(srv.poll(t)[0] == abi.HS_REQ_GONE for t in tickets)


def test_oversize_request_denied_and_bad_input_rejected(hs):
    spec = request_spec(5000, 32, 7)
    with hs.Context() as ctx, hs.Server(ctx, budget_bytes=1 << 20) as srv:
        with pytest.raises(hs.HairSimError) as e:
            submit(srv, spec, 10)
        assert e.value.status == abi.HS_ERR_ADMISSION_DENIED
        small = request_spec(64, 8, 8)
        small["sim"].root_mode = abi.HS_ROOT_EXPLICIT
        with pytest.raises(hs.HairSimError) as e:
            submit(srv, small, 10)
        assert e.value.status == abi.HS_ERR_UNSUPPORTED
        small["sim"].root_mode = abi.HS_ROOT_SKINNED   # without influences
        with pytest.raises(hs.HairSimError) as e:
            submit(srv, small, 10)
        assert e.value.status == abi.HS_ERR_INVALID_ARG
        with pytest.raises(hs.HairSimError):
            srv.tick(0.0)


def test_poll_states_and_collect(hs):
    spec = request_spec(256, 8, 9)
    with hs.Context() as ctx, hs.Server(ctx, budget_bytes=1 << 26) as srv:
        t = submit(srv, spec, 3, keep=True)
        assert srv.poll(t) == (abi.HS_REQ_QUEUED, 0)
        with pytest.raises(hs.HairSimError):
            srv.collect(t)
        srv.tick(DT)                       # admitted, set up
        assert srv.poll(t)[0] == abi.HS_REQ_RESIDENT
        for _ in range(3):
            srv.tick(DT)
        assert srv.poll(t) == (abi.HS_REQ_DONE, 3)
        p, v = srv.collect(t)
        assert np.isfinite(p).all() and p.shape == (256, 8, 4)
        assert srv.poll(t)[0] == abi.HS_REQ_GONE


# ---- per-tick inputs: moving spheres, rigid and skinned roots -------------

AXIS = np.array([0.3, 0.8, 0.52])


def rigid_m(f):
    return scenarios.rigid_motion((f + 1) * DT, AXIS / np.linalg.norm(AXIS), 25.0, 0.2, 0.3)


def moving_spheres(base, f):
    s = base.copy()
    s[:, 0] += np.float32(0.1 * math.sin(3.0 * (f + 1) * DT))
    return s


def moving_specs():
    rigid = request_spec(1500, 24, 401)
    rigid["sim"].root_mode = abi.HS_ROOT_RIGID
    sk = scenarios.skinned(ns=2048, npoints=16, nspheres=8, substeps=4)
    skinned = dict(roots=sk.roots, normals=sk.normals, strand=sk.strand, sim=sk.sim, spheres=sk.spheres_at(0),
                   lengths=None, wind=(0.0, 0.0, 0.0), swing_amp=0.0, swing_omega=0.0,
                   skin=(sk.bones, sk.weights), rig=sk)
    pinned = request_spec(900, 16, 402)
    return {"rigid": rigid, "skinned": skinned, "pinned": pinned}


def submit_moving(srv, spec, frames):
    skin = spec.get("skin")
    return srv.submit(spec["roots"], spec["normals"], spec["strand"], spec["sim"], frames, spheres=spec["spheres"],
                      wind=spec["wind"], swing_amp=spec["swing_amp"], swing_omega=spec["swing_omega"], keep=True,
                      lengths=spec["lengths"], skin_bones=None if skin is None else skin[0],
                      skin_weights=None if skin is None else skin[1])


def feed(srv, live):
    """Before a tick: each live groom gets the inputs of its own next frame."""
    for name, (t, spec) in live.items():
        state, f = srv.poll(t)
        if state not in (abi.HS_REQ_QUEUED, abi.HS_REQ_RESIDENT):
            continue
        if name == "rigid":
            srv.set_root_transform(t, rigid_m(f))
            srv.set_spheres(t, moving_spheres(spec["spheres"], f))
        elif name == "skinned":
            srv.set_bone_matrices(t, spec["rig"].rig.matrices(f + 1))
            srv.set_spheres(t, spec["rig"].spheres_at(f + 1))
        else:
            srv.set_spheres(t, moving_spheres(spec["spheres"], f))


def test_moving_inputs_same_alone_and_in_the_mix(hs):
    """Spheres moved, rigid roots transformed and bone palettes changed by
    ticket before every tick, each as a function of the groom's own frame:
    every result is the same alone and in a mix of other requests arriving
    and leaving, and the rigid groom matches the oracle."""
    specs = moving_specs()
    frames = 20
    with hs.Context() as ctx:
        alone = {}
        for name, spec in specs.items():
            with hs.Server(ctx, budget_bytes=1 << 30) as srv:
                live = {name: (submit_moving(srv, spec, frames), spec)}
                for _ in range(frames + 5):
                    feed(srv, live)
                    srv.tick(DT)
                alone[name] = srv.collect(live[name][0])
        with hs.Server(ctx, budget_bytes=1 << 30) as srv:
            others = [request_spec(400 + 600 * k, [8, 16, 32][k % 3], 500 + k) for k in range(5)]
            tickets = [submit(srv, others[0], 30), submit(srv, others[1], 6)]
            live = {}
            for k, (name, spec) in enumerate(specs.items()):
                feed(srv, live)
                srv.tick(DT)
                live[name] = (submit_moving(srv, spec, frames), spec)
                tickets.append(submit(srv, others[2 + k], 8 + 4 * k))
            for _ in range(200):
                if all(srv.poll(t)[0] in (abi.HS_REQ_DONE, abi.HS_REQ_GONE) for t, _ in live.values()):
                    break
                feed(srv, live)
                srv.tick(DT)
            mixed = {name: srv.collect(t) for name, (t, _) in live.items()}
    for name in specs:
        util.assert_bit_equal(mixed[name][0], alone[name][0], f"{name}: positions alone vs mix")
        util.assert_bit_equal(mixed[name][1], alone[name][1], f"{name}: velocities alone vs mix")
    # The rigid groom against the oracle, frame by frame.
    spec = specs["rigid"]
    sp = spec["strand"]
    p, v = oracle.init(spec["roots"], spec["normals"], sp, dtype=np.float32, lengths=spec["lengths"])
    rest = p[:, 0, :3].copy()
    dt32 = float(np.float32(DT))
    amp, om = float(np.float32(1.5)), float(np.float32(0.7))
    for f in range(frames):
        t = (f + 1) * dt32
        w = np.array([np.float32(0.0) + np.float32(amp * math.sin(om * t)), 0.0, 0.5], np.float32)
        oracle.frame(p, v, spec["sim"], DT, seed=int(sp.seed), wind=w, spheres=moving_spheres(spec["spheres"], f),
                     root_targets=oracle.rigid_targets(rest, rigid_m(f), np.float32))
    util.assert_bit_equal(alone["rigid"][0], p, "served rigid groom vs oracle")


def test_setters_reject_what_the_request_does_not_take(hs):
    spec = request_spec(128, 8, 11)
    with hs.Context() as ctx, hs.Server(ctx, budget_bytes=1 << 26) as srv:
        t = submit(srv, spec, 2)
        with pytest.raises(hs.HairSimError) as e:
            srv.set_root_transform(t, np.eye(4, dtype=np.float32).reshape(16))   # pinned roots
        assert e.value.status == abi.HS_ERR_UNSUPPORTED
        with pytest.raises(hs.HairSimError) as e:
            srv.set_bone_matrices(t, np.eye(4, dtype=np.float32).reshape(1, 16))
        assert e.value.status == abi.HS_ERR_UNSUPPORTED
        srv.set_spheres(t, spec["spheres"][:2])                                  # queued: kept
        for _ in range(4):
            srv.tick(DT)
        with pytest.raises(hs.HairSimError) as e:
            srv.set_spheres(t, spec["spheres"])                                  # done and gone
        assert e.value.status == abi.HS_ERR_INVALID_ARG
