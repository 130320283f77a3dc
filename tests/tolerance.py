"""FP32-vs-FP64 tolerance checks of the benchmark configurations.

The tolerances (one step <= 1e-5 x strand length, segment length <= 1e-5
relative, 60-frame drift <= 1e-3 x strand length) compare the library's FP32
arithmetic with the FP64 oracle (DFTL mode in world coordinates, Mueller et
al.'s algorithm as written) from the same state and inputs. Strands are
independent, so a configuration is checked on sampled blocks of strands.

Which strands a bound can hold for is decided from the FP64 runs alone,
never from the FP32 result:
  * contact: the FP64 trajectory with the configuration's spheres differs
    from the FP64 trajectory without them (some push-out happened). Push-out
    is discontinuous (a point just inside or just outside a sphere), so
    contact strands get a looser, separately stated bound;
  * ill-conditioned: the FP64 trajectory amplifies a 1e-7 perturbation of
    the initial positions past 1e-4 x strand length (x1000) within the
    frames run. Upright strands (an unstable equilibrium) and strands whose
    roots accelerate faster than gravity do this without any sphere; no
    FP32 arithmetic can track FP64 there, so the 60-frame bound covers the
    well-conditioned, contact-free strands and the covered fraction is
    asserted too;
  * for one frame, ill-conditioned: one FP64 frame amplifies a 1e-7
    perturbation of its start past 1e-5 x strand length (x100): a strand
    folded back on itself (consecutive segments antiparallel) or balanced
    upright. The one-step and segment bounds cover the other contact-free
    strands; every strand is held to CONTACT_ONE_STEP_TOL for one frame.
"""
from __future__ import annotations

import dataclasses

import numpy as np

import oracle
from barbu_gb300 import scenarios
from tests import util

ONE_STEP_TOL = 1e-5
SEGMENT_TOL = 1e-5
DRIFT_TOL = 1e-3
# Contact strands, one frame: push-out moves a point to the sphere surface
# along p - c, which is ill-conditioned for points deep inside a sphere.
CONTACT_ONE_STEP_TOL = 1e-3
PERTURBATION = 1e-7
ILL_CONDITIONED = 1e-4
STEP_ILL_CONDITIONED = 1e-5
DT = 1 / 60


def blocks(ns: int, nblocks: int, size: int, seed: int = 11) -> list[tuple[int, int]]:
    """Disjoint blocks (start, length) of consecutive strands, plus the last
    partial warp of the groom."""
    size = min(size, ns)
    rng = np.random.default_rng(seed)
    nb = min(nblocks, max(1, ns // size))
    starts = np.sort(rng.choice(ns // size, size=nb, replace=False)) * size
    out = [(int(s), size) for s in starts]
    tail = ns % 32 or 32
    if ns > size and all(s + k <= ns - tail for s, k in out):
        out.append((ns - tail, tail))
    return out


class Feed:
    """Per-frame inputs of one configuration (frame f is 0-based: its inputs
    are those of time (f + 1) dt)."""

    def __init__(self, spec):
        self.spec = spec
        self.skinned = isinstance(spec, scenarios.SkinnedSpec)

    def gpu(self, groom, f: int):
        s = self.spec
        if self.skinned:
            groom.set_bone_matrices(s.rig.matrices(f + 1))
            groom.set_spheres(s.spheres_at(f + 1))
            return
        t = (f + 1) * DT
        if s.wind:
            groom.set_wind(scenarios.wind_at(t))
        m = s.transform(t)
        if m is not None:
            groom.set_root_transform(m)
        groom.set_spheres(s.spheres_at(t))

    def oracle_args(self, f: int, b: int, k: int, dtype, spheres: bool = True) -> dict:
        s = self.spec
        if self.skinned:
            dq = oracle.matrix_to_dual_quat(s.rig.matrices(f + 1))
            tg = oracle.skin_targets(s.roots[b:b + k], s.bones[b:b + k], s.weights[b:b + k], dq, dtype=dtype)
            return dict(seed=int(s.strand.seed), spheres=s.spheres_at(f + 1) if spheres else None,
                        root_targets=tg, strand_base=b)
        t = (f + 1) * DT
        m = s.transform(t)
        tg = oracle.rigid_targets(s.roots[b:b + k], m, dtype) if m is not None else None
        return dict(seed=int(s.strand.seed), wind=scenarios.wind_at(t) if s.wind else None,
                    spheres=s.spheres_at(t) if spheres else None, root_targets=tg, strand_base=b)


@dataclasses.dataclass
class Report:
    one_step: np.ndarray          # per strand, frame 1 from the initial state
    one_step_mid: np.ndarray      # per strand, frame `mid` from the FP32 state of frame mid - 1
    segment: np.ndarray           # per strand, max relative segment-length error of those two frames
    contact_step: np.ndarray      # contact during frame 1 or frame `mid`
    step_ill: np.ndarray          # frame 1 or frame `mid` ill-conditioned
    drift: np.ndarray             # per strand, after the last frame
    contact: np.ndarray           # contact in any frame
    ill: np.ndarray               # ill-conditioned
    lengths: np.ndarray

    def summary(self) -> dict:
        free_step = ~self.contact_step & ~self.step_ill
        covered = ~self.contact & ~self.ill
        f = lambda a: float(a.max()) if a.size else 0.0
        return dict(strands=int(self.drift.size),
                    one_step_free=f(np.maximum(self.one_step, self.one_step_mid)[free_step]),
                    one_step_other=f(np.maximum(self.one_step, self.one_step_mid)[~free_step]),
                    step_covered=float(free_step.mean()),
                    segment_free=f(self.segment[free_step]),
                    drift_covered=f(self.drift[covered]),
                    covered=float(covered.mean()), contact=float(self.contact.mean()),
                    ill=float((self.ill & ~self.contact).mean()),
                    drift_other=f(self.drift[~covered]))

    def long_run(self) -> dict:
        """Drift on the covered strands after a configuration's specified
        run: median, 99th percentile, largest."""
        covered = ~self.contact & ~self.ill
        d = self.drift[covered]
        q = (lambda x: float(np.quantile(d, x))) if d.size else (lambda x: 0.0)
        return dict(covered=float(covered.mean()), median=q(0.5), p99=q(0.99), max=q(1.0))

    def check_long(self, min_covered: float, min_step_covered: float = 0.0):
        """A specified run longer than 60 frames: the one-frame bounds as
        check(); the drift bound on 99 % of the covered strands, and ten times
        it on all of them. FP32 rounding enters every frame: over hundreds of
        frames a few strands that swing through an unstable configuration
        separate transiently from FP64 although a perturbation of the initial
        state alone does not grow there (measured on a batched groom: median
        drift 3e-6 from frame 30 to 300, largest 1.5e-4 at frame 120 and
        3.0e-3 at 300)."""
        free_step = ~self.contact_step & ~self.step_ill
        step = np.maximum(self.one_step, self.one_step_mid)
        assert free_step.mean() >= min_step_covered, self.summary()
        assert step[free_step].max(initial=0) <= ONE_STEP_TOL, self.summary()
        assert self.segment[free_step].max(initial=0) <= SEGMENT_TOL, self.summary()
        assert step.max(initial=0) <= CONTACT_ONE_STEP_TOL, self.summary()
        lr = self.long_run()
        assert lr["covered"] >= min_covered, lr
        assert lr["p99"] <= DRIFT_TOL, lr
        assert lr["max"] <= 10 * DRIFT_TOL, lr

    def check(self, min_covered: float, min_step_covered: float = 0.0):
        free_step = ~self.contact_step & ~self.step_ill
        step = np.maximum(self.one_step, self.one_step_mid)
        assert free_step.mean() >= min_step_covered, self.summary()
        assert step[free_step].max(initial=0) <= ONE_STEP_TOL, self.summary()
        assert self.segment[free_step].max(initial=0) <= SEGMENT_TOL, self.summary()
        assert step.max(initial=0) <= CONTACT_ONE_STEP_TOL, self.summary()
        covered = ~self.contact & ~self.ill
        assert covered.mean() >= min_covered, self.summary()
        assert self.drift[covered].max(initial=0) <= DRIFT_TOL, self.summary()


def _err(a, b, lengths):
    return np.linalg.norm(a[..., :3].astype(np.float64) - b[..., :3], axis=-1).max(axis=1) / lengths


def _seg_err(a, b):
    sa, sb = util.segment_lengths(a), util.segment_lengths(b)
    return (np.abs(sa - sb) / np.maximum(sb, 1e-30)).max(axis=1)


def evaluate(feed: Feed, blk: list[tuple[int, int]], states: dict[int, np.ndarray], frames: int, mid: int,
             sim=None) -> Report:
    """states[f]: FP32 positions and velocities (ns_sample, N, 8: pos then
    vel) of the sampled strands after frame f (0: the initial state), at
    f in {0, 1, mid - 1, mid, frames}. Runs the FP64 oracle from the same
    initial state (with and without spheres, and perturbed) and one FP64
    frame from the FP32 state of frame mid - 1."""
    sim = sim or feed.spec.sim
    s0 = states[0]
    q = s0[..., :4].astype(np.float64).copy()
    w = s0[..., 4:].astype(np.float64).copy()
    q0, w0 = q.copy(), w.copy()
    rng = np.random.default_rng(3)
    qp, wp = q.copy(), w.copy()
    qp[:, 1:, :3] += PERTURBATION * rng.standard_normal(qp[:, 1:, :3].shape)
    L = util.strand_lengths(s0[..., :4])
    n = len(L)
    contact = np.zeros(n, bool)
    contact_step = np.zeros(n, bool)
    step_ill = np.zeros(n, bool)
    cond = np.zeros(n)
    one_step = one_mid = segment = None
    bounds = []
    o = 0
    for b, k in blk:
        bounds.append((b, k, o))
        o += k
    for f in range(frames):
        if f == mid - 1:
            # One FP64 frame from the FP32 state of frame mid - 1, with and
            # without spheres.
            m = states[mid - 1][..., :4].astype(np.float64).copy()
            mv = states[mid - 1][..., 4:].astype(np.float64).copy()
            m0, mv0 = m.copy(), mv.copy()
            mp, mvp = m.copy(), mv.copy()
            mp[:, 1:, :3] += PERTURBATION * rng.standard_normal(mp[:, 1:, :3].shape)
            for b, k, o in bounds:
                oracle.frame(m[o:o + k], mv[o:o + k], sim, DT, **feed.oracle_args(f, b, k, np.float64))
                oracle.frame(m0[o:o + k], mv0[o:o + k], sim, DT, **feed.oracle_args(f, b, k, np.float64, False))
                oracle.frame(mp[o:o + k], mvp[o:o + k], sim, DT, **feed.oracle_args(f, b, k, np.float64))
            one_mid = _err(states[mid][..., :4], m, L)
            seg_mid = _seg_err(states[mid][..., :4], m)
            contact_step |= (m != m0).any(axis=(1, 2))
            step_ill |= _err(mp, m, L) > STEP_ILL_CONDITIONED
        for b, k, o in bounds:
            oracle.frame(q[o:o + k], w[o:o + k], sim, DT, **feed.oracle_args(f, b, k, np.float64))
            oracle.frame(q0[o:o + k], w0[o:o + k], sim, DT, **feed.oracle_args(f, b, k, np.float64, False))
            oracle.frame(qp[o:o + k], wp[o:o + k], sim, DT, **feed.oracle_args(f, b, k, np.float64))
        touched = (q != q0).any(axis=(1, 2))
        contact |= touched
        cond = np.maximum(cond, np.linalg.norm(qp[..., :3] - q[..., :3], axis=-1).max(axis=1) / L)
        if f == 0:
            one_step = _err(states[1][..., :4], q, L)
            segment = _seg_err(states[1][..., :4], q)
            contact_step |= touched
            step_ill |= cond > STEP_ILL_CONDITIONED
    return Report(one_step=one_step, one_step_mid=one_mid, segment=np.maximum(segment, seg_mid),
                  contact_step=contact_step, step_ill=step_ill, drift=_err(states[frames][..., :4], q, L), contact=contact,
                  ill=cond > ILL_CONDITIONED, lengths=L)


def oracle_states(feed: Feed, blk, frames: int, mid: int) -> dict[int, np.ndarray]:
    """The FP32 oracle's states of the sampled strands (the library's
    contract, bit for bit), for runs without a GPU."""
    s = feed.spec
    p, v = oracle.init(s.roots, s.normals, s.strand, dtype=np.float32, lengths=s.lengths)
    p = np.concatenate([p[b:b + k] for b, k in blk])
    v = np.concatenate([v[b:b + k] for b, k in blk])
    keep = {0, 1, mid - 1, mid, frames}
    out = {0: np.concatenate([p, v], axis=-1)}
    for f in range(frames):
        o = 0
        for b, k in blk:
            oracle.frame(p[o:o + k], v[o:o + k], s.sim, DT, **feed.oracle_args(f, b, k, np.float32))
            o += k
        if f + 1 in keep:
            out[f + 1] = np.concatenate([p, v], axis=-1)
    return out
