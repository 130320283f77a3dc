"""Benchmark of the hair-strand simulation step on GB300.

Metric: strand-point substeps/s = strands x points x substeps x frames / s,
batched (and served) against the plain per-groom launch path.
A step is one frame: every strand of the workload advanced by S substeps.

Workloads (seeded synthetic grooms, barbu_gb300/scenarios.py):
  batched  64 grooms, strand counts log-uniform in [1,024, 131,072], points
           per strand from {8, 16, 24, 32}, rigid root motion per groom,
           1-16 spheres, 8 substeps (default; the metric's batched case).
           Ours: hs_update_many, autotuned, one CUDA graph launch per frame.
           Also timed: the plain path, one hs_update launch per groom.
  large    262,144 strands x 32 points, 16 spheres, wind, 8 substeps,
           one groom through hs_update.
  plain    4,096 strands x 16 points, 1 moving sphere, 4 substeps.
  With the batched workload the line also carries `workloads`: the plain,
  large and skinned configurations measured the same way in the same run
  (device-timed value, roofline, e2e, a shorter CPU sample), and `served`: the served
  stream (hs_server_*) with Poisson arrivals at 20, 100 and 500 grooms per
  simulated second, an 8 GB admission budget, p50/p99 tick latency and
  throughput, and a fixed population of 64 resident grooms.

Our arm (default):
  value     device-timed: K frames back to back, state resident in HBM (all
            workloads but `plain` hold more than the 129 MB L2; `plain` is
            L2-resident by nature and says so), CUDA events on the library's
            stream, max over ranks.
  e2e       the same frames through the public API with host buffers: per
            frame the inputs (root transforms, wind, spheres) go in from host
            memory and every position the renderer consumes comes back to
            pinned host memory; the median of three timed runs of each loop
            after an untimed one (all three under `runs`).
  roofline  the step against measured HBM bandwidth: algorithmic bytes = 64
            B per control point per frame (float4 position and velocity, read
            once and written once), over the device time of one frame.
            `traffic` (DRAM bytes) and `issue` (warp instructions) come from
            the committed ncu summary in profiles/; each records the hash of
            the kernel sources it was captured at, and a mismatch with the
            sources being run marks them stale (traffic null, issue.stale).
  cpu_baseline  the oracle's FP32 instantiation, OpenMP over all host
            cores, on the same workload for about 10 s (rank 0, N = 1).
--impl reference: the oracle's FP32 restatement of the reference step
(the reference is a GLSL compute pass with no CPU implementation and no
graphics stack here), timed on the host cores on the same workload.

Multi-GPU (torchrun): each rank advances its own replica of the workload
(weak scaling, no collective on the data path); the barrier and the max of
the per-rank times use torch.distributed.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
BYTES_PER_POINT = 64
METRIC = "strand-point substeps/s"
DT = 1.0 / 60.0
E2E_RUNS = 3  # timed runs of each end-to-end loop; the median is reported


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["batched", "large", "plain", "skinned"], default="batched")
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-tess", action="store_true")
    ap.add_argument("--no-others", action="store_true",
                    help="batched: leave out the single-groom configurations (plain, large, skinned)")
    ap.add_argument("--served-ticks", type=int, default=240)
    ap.add_argument("--served-budget-gb", type=float, default=8.0)
    ap.add_argument("--strands", type=int, default=None,
                    help="strands of a single-groom workload (default: the workload's own size)")
    ap.add_argument("--contract", choices=["exact", "fast"], default="fast",
                    help="arithmetic contract of the DFTL chain link (hs_contract) of the line's grooms")
    ap.add_argument("--no-alt-contract", action="store_true",
                    help="batched: leave out the batched workload under the other contract")
    return ap.parse_args()


# ---- workloads -------------------------------------------------------------

def rigid_series(spec, frames: int, start: int = 0) -> np.ndarray:
    """Column-major root transforms of one groom for frames [start, start+frames)."""
    from barbu_gb300 import scenarios
    return np.stack([scenarios.rigid_motion((start + f + 1) * DT, spec.axis, spec.omega_deg, spec.amp, spec.phase)
                     for f in range(frames)])


L2_BYTES = 129 * 1000 * 1000  # GB300 L2 (nominal)


def l2_note(points):
    """How the timed frames relate to the L2: the state is 32 B per point
    (position and velocity), read and written once per frame."""
    state = 32 * int(points)
    if state > L2_BYTES:
        return f"state ({state / 1e6:.0f} MB at 32 B/point) exceeds the 129 MB L2; no flush"
    return f"L2-resident ({state / 1e6:.1f} MB of state) by nature; no flush"


class Workload:
    name = ""
    contract = "exact"

    def __init__(self, specs):
        self.specs = specs

    @property
    def points_per_frame(self) -> int:
        return sum(s.nstrands * s.npoints * int(s.sim.substeps) for s in self.specs)

    @property
    def points(self) -> int:
        return sum(s.nstrands * s.npoints for s in self.specs)

    def config(self, world):
        raise NotImplementedError

    # Host side of the end-to-end loop: one pinned buffer per groom,
    # (x, y, z, rest) or (x, y, z) per point, strand-major.
    def host_buffers(self, torch, comps=4):
        """One pinned host buffer holding every groom's strand-major frame,
        comps floats a point, in list order; and its size in bytes."""
        total = sum(s.nstrands * s.npoints * comps for s in self.specs)
        t = torch.empty(total, dtype=torch.float32, pin_memory=True).numpy()
        return [t], t.nbytes

    def views(self, flat, comps):
        out, at = [], 0
        for s in self.specs:
            size = s.nstrands * s.npoints * comps
            out.append(flat[at:at + size].reshape(s.nstrands, s.npoints, comps))
            at += size
        return out

    def readback(self, host):
        """Blocking: one hs_readback per groom."""
        for g, h in zip(self.readback_grooms(), self.views(host[0], 4)):
            g.readback(h)

    def queue_readback(self, host, comps):
        """Asynchronous: a groom alone through its own call, several through
        hs_readback_many_async (one copy for all)."""
        grooms = self.readback_grooms()
        if len(grooms) == 1:
            view = self.views(host[0], comps)[0]
            (grooms[0].readback_xyz_async if comps == 3 else grooms[0].readback_async)(view)
        else:
            self.ctx.readback_many_async(grooms, host[0], comps=comps, handles=getattr(self, "handles", None))

    def readback_async(self, host):
        self.queue_readback(host, 4)

    def readback_xyz_async(self, host):
        self.queue_readback(host, 3)


class Single(Workload):
    def __init__(self, name, spec):
        super().__init__([spec])
        self.name = name
        self.spec = spec

    def setup(self, ctx, frames):
        from barbu_gb300 import scenarios
        s = self.spec
        self.g = ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths)
        self.g.set_spheres(s.spheres)
        from barbu_gb300 import abi
        self.mapping = ("lane groups (a lane per substep)" if self.g.mapping() == abi.HS_MAPPING_LANES
                        else "a thread per strand")
        # Every frame's inputs up front, as float32 arrays the calls take as they are.
        ts = [(f + 1) * DT for f in range(frames + 1)]
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        self.W = [f32(scenarios.wind_at(t)) for t in ts] if s.wind else None
        self.M = [f32(s.transform(t)) for t in ts] if s.moving_roots != "none" else None
        self.S = [f32(s.spheres_at(t)) for t in ts] if s.moving_roots == "translate_x" else None

    def inputs(self, f):
        if self.W is not None:
            self.g.set_wind(self.W[f % len(self.W)])
        if self.M is not None:
            self.g.set_root_transform(self.M[f % len(self.M)])
        if self.S is not None:
            self.g.set_spheres(self.S[f % len(self.S)])

    def step(self, ctx):
        self.g.update(DT)

    def h2d_bytes(self):
        s = self.spec
        return 4 * ((3 if s.wind else 0) + (16 if s.moving_roots != "none" else 0)
                    + (4 * s.spheres.shape[0] if s.moving_roots == "translate_x" else 0))

    def readback_grooms(self):
        return [self.g]

    def destroy(self):
        self.g.destroy()

    def config(self, world):
        s = self.spec
        return {"workload": self.name, "grooms": 1, "strands": s.nstrands, "points_per_strand": s.npoints,
                "substeps": int(s.sim.substeps), "spheres": int(s.spheres.shape[0]), "mode": "dftl",
                "dt": DT, "replicas": world, "path": "plain (hs_update, one launch per frame)",
                "l2": l2_note(self.points)}


class Skinned(Workload):
    """One groom whose roots are skinned to an animated bone chain: the bone
    matrices and the bone-attached spheres of every frame are computed up
    front and fed through hs_set_bone_matrices / hs_set_spheres."""
    name = "skinned"

    def __init__(self, spec):
        super().__init__([spec])
        self.spec = spec

    def setup(self, ctx, frames):
        s = self.spec
        self.g = ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths)
        self.g.set_skin(s.bones, s.weights)
        self.M = [s.rig.matrices(f + 1) for f in range(frames + 1)]
        self.S = [s.spheres_at(f + 1) for f in range(frames + 1)]
        # The mapping is resolved against a complete groom: bones loaded.
        self.g.set_bone_matrices(self.M[0])
        from barbu_gb300 import abi
        self.mapping = ("lane groups (a lane per substep)" if self.g.mapping() == abi.HS_MAPPING_LANES
                        else "a thread per strand")

    def inputs(self, f):
        self.g.set_bone_matrices(self.M[f % len(self.M)])
        self.g.set_spheres(self.S[f % len(self.S)])

    def step(self, ctx):
        self.g.update(DT)

    def h2d_bytes(self):
        return int(self.M[0].nbytes + self.S[0].nbytes)

    def readback_grooms(self):
        return [self.g]

    def destroy(self):
        self.g.destroy()

    def config(self, world):
        s = self.spec
        return {"workload": "skinned", "grooms": 1, "strands": s.nstrands, "points_per_strand": s.npoints,
                "substeps": int(s.sim.substeps), "spheres": int(len(s.sphere_rest)), "mode": "dftl",
                "roots": "dual-quaternion skinned, 4-bone chain, 2 weights per root, <= 2 deg/frame random walks",
                "mesh": "cylinder r 0.5 h 2, 8 rings x 64 segments", "dt": DT, "replicas": world,
                "path": "plain (hs_update, one launch per frame, skinning fused into the step)",
                "l2": l2_note(self.points)}


class Batched(Workload):
    name = "batched"

    def setup(self, ctx, frames):
        self.grooms = [ctx.groom(s.roots, s.normals, s.strand, s.sim, lengths=s.lengths) for s in self.specs]
        for g, s in zip(self.grooms, self.specs):
            g.set_spheres(s.spheres)
        self.handles = ctx.handles_of(self.grooms)
        # Root transforms of every groom for every frame, computed up front.
        self.M = np.ascontiguousarray(np.stack([rigid_series(s, frames) for s in self.specs], axis=1),
                                      dtype=np.float32)  # [frames, grooms, 16]

    def inputs(self, f):
        from barbu_gb300 import hairsim  # noqa: F401
        self.ctx.set_root_transforms(self.grooms, self.M[f % len(self.M)], handles=self.handles)

    def step(self, ctx):
        ctx.update_many(self.grooms, DT, handles=self.handles)

    def plain_step(self, f):
        m = self.M[f % len(self.M)]
        for i, g in enumerate(self.grooms):
            g.set_root_transform(m[i])
            g.update(DT)

    def h2d_bytes(self):
        return 4 * 16 * len(self.specs)

    def readback_grooms(self):
        return self.grooms

    def destroy(self):
        for g in self.grooms:
            g.destroy()

    def config(self, world):
        ns = [s.nstrands for s in self.specs]
        npts = [s.npoints for s in self.specs]
        return {"workload": "batched", "grooms": len(self.specs), "strands": int(sum(ns)),
                "strands_min": int(min(ns)), "strands_max": int(max(ns)),
                "points": int(self.points), "points_per_strand": sorted(set(npts)),
                "substeps": int(self.specs[0].sim.substeps),
                "spheres_per_groom": [int(min(s.spheres.shape[0] for s in self.specs)),
                                      int(max(s.spheres.shape[0] for s in self.specs))],
                "mode": "dftl", "roots": "rigid motion per groom", "dt": DT, "replicas": world,
                "path": "batched (hs_update_many: autotuned persistent kernels, one CUDA graph per frame)",
                "l2": l2_note(self.points)}


class ServedShapes:
    """Groom shapes of the served stream, drawn from the batched workload's
    size distribution: strand counts log-uniform over [1,024, 131,072]
    (12 log-spaced classes), points per strand from {8, 16, 24, 32}, roots
    on a sphere, lengths U[0.3, 0.8], 1-16 spheres, wind with a swing, pinned
    roots. Each request draws a class and a point count uniformly, a
    lifetime of U[30, 300] frames, and runs 4 substeps."""

    def __init__(self, classes: int = 12, seed: int = 0xBA5B0 + 4, lo: int = 1024, hi: int = 131072,
                 points=(8, 16, 24, 32), contract: int = 0):
        from barbu_gb300 import abi, scenarios
        self.abi = abi
        self.points = tuple(points)
        self.contract = contract
        sizes = np.unique(np.round(np.exp(np.linspace(np.log(lo), np.log(hi), classes))).astype(int))
        self.shapes = []
        for k, ns in enumerate(sizes):
            roots, normals = scenarios.sphere_roots(int(ns), seed + k)
            rng = np.random.default_rng([seed, k])
            lengths = rng.uniform(0.3, 0.8, int(ns)).astype(np.float32)
            spheres = scenarios.shell_spheres(int(rng.integers(1, 17)), seed + k)
            self.shapes.append((roots, normals, lengths, spheres))

    def request(self, rng, keep=False):
        abi = self.abi
        k = int(rng.integers(len(self.shapes)))
        roots, normals, lengths, spheres = self.shapes[k]
        npoints = int(rng.choice(self.points))
        sp = abi.strand_params(npoints, abi.HS_LENGTH_TOTAL, 0.5, 0.0, int(rng.integers(1 << 30)))
        sim = abi.sim_params_dftl(substeps=4, damping=0.9, wind_jitter=0.2, contract=self.contract)
        frames = int(rng.integers(30, 301))
        return dict(roots=roots, normals=normals, strand=sp, sim=sim, frames=frames, spheres=spheres,
                    wind=(0.0, 0.0, 0.5), swing_amp=1.5, swing_omega=0.7, keep=keep, lengths=lengths)


def run_served(ctx, shapes, rate, ticks, warm, budget, seed=7):
    """Poisson arrivals at `rate` per simulated second; returns tick stats."""
    from barbu_gb300 import hairsim
    rng = np.random.default_rng([seed, int(rate)])
    srv = hairsim.Server(ctx, budget_bytes=budget)
    next_arrival = rng.exponential(1.0 / rate)
    lat, work, resident, queued = [], 0, [], []
    wall = 0.0
    submitted = 0
    for k in range(warm + ticks):
        t = k * DT
        while next_arrival <= t:
            q = shapes.request(rng)
            srv.submit(**q)
            submitted += 1
            next_arrival += rng.exponential(1.0 / rate)
        st = srv.tick(DT)
        if k >= warm:
            lat.append(st.tick_ms)
            work += st.point_substeps
            wall += st.tick_ms * 1e-3
            resident.append(st.advanced)
            queued.append(st.queued)
    srv.close()
    lat = np.array(lat)
    return {"rate_per_s": rate, "ticks": ticks, "warmup_ticks": warm, "requests": submitted,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()), "value": work / wall if wall > 0 else 0.0,
            "resident_mean": float(np.mean(resident)), "queued_at_end": int(queued[-1])}


def run_fixed(ctx, shapes, n, ticks, warm, budget, seed=11):
    """n grooms resident the whole time (lifetimes longer than the run)."""
    from barbu_gb300 import hairsim
    rng = np.random.default_rng([seed, n])
    srv = hairsim.Server(ctx, budget_bytes=budget)
    for _ in range(n):
        q = shapes.request(rng)
        q["frames"] = warm + ticks + 10
        srv.submit(**q)
    lat, work, wall, adv = [], 0, 0.0, []
    for k in range(warm + ticks + 1):
        st = srv.tick(DT)
        if k > warm:
            lat.append(st.tick_ms)
            work += st.point_substeps
            wall += st.tick_ms * 1e-3
            adv.append(st.advanced)
    srv.close()
    lat = np.array(lat)
    return {"resident_grooms": int(np.min(adv)), "ticks": ticks, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()), "value": work / wall}


def run_tess(torch, ctx, stream, passes=20, warm=3):
    """The tessellation stream pass on the plain groom (4,096 strands x 16
    points on a sphere, its convex-hull triangles), reference settings (3
    instances, 2 lines, 16 subsegments): output vertices per second and the
    write bandwidth (16 B per vertex)."""
    from barbu_gb300 import abi, hairsim, scenarios
    try:
        from scipy.spatial import ConvexHull
    except ImportError:
        return {"unavailable": "scipy is not installed (triangulation of the roots)"}
    spec = scenarios.plain()
    faces = ConvexHull(spec.roots.astype(np.float64)).simplices.astype(np.uint32)
    rng = np.random.default_rng(5)
    tangents = rng.uniform(-0.1, 0.1, (spec.nstrands, spec.npoints, 4)).astype(np.float32)
    rand = rng.random(abi.HS_TESS_RANDOM_SIZE).astype(np.float32)
    g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim)
    g.tess_setup(faces, tangents, rand)
    p = hairsim.tess_params_reference()
    for _ in range(warm):
        count = g.tess_stream(p)
    ms, _ = timed_frames(torch, ctx, stream, passes, 0, lambda f: g.tess_stream(p), "timed_tess")
    g.destroy()
    per = ms / passes
    return {"triangles": int(len(faces)), "strands": spec.nstrands, "points_per_strand": spec.npoints,
            "instances": int(p.ninstances), "lines": int(p.nlines), "subsegments": int(p.nsubsegments),
            "vertices_per_pass": int(count), "ms_per_pass": per, "vertices_per_s": count / (per * 1e-3),
            "write_gbs": 16.0 * count / (per * 1e-3) / 1e9}


CONTRACTS = {
    "fast": "fast: the chain link's and the push-out normal's reciprocal square roots from the GPU's "
            "rsqrt.approx (the hardware inversesqrt a GLSL compute pass gets); FP32 throughout, held to the "
            "FP64 tolerances",
    "exact": "exact: the chain link's reciprocal square root restated from IEEE add, multiply and fma "
             "(< 1 ulp), so that the GPU and the FP32 oracle agree bit for bit",
}


def make_workload(name, strands=None, contract="exact") -> Workload:
    """The named workload; `strands` shrinks a single-groom workload (a
    smaller case of the same kernel, for profiler captures); `contract`:
    the DFTL chain link's arithmetic (hs_contract) of every groom."""
    from barbu_gb300 import abi, scenarios
    kw = {} if strands is None else {"ns": int(strands)}
    if name == "batched":
        if strands is not None:
            raise SystemExit("--strands applies to the single-groom workloads")
        wl = Batched(scenarios.batched())
    elif name == "large":
        wl = Single("large", scenarios.large(**kw))
    elif name == "skinned":
        wl = Skinned(scenarios.skinned(**kw))
    else:
        wl = Single("plain", scenarios.plain(**kw))
    for s in wl.specs:
        s.sim.contract = abi.HS_CONTRACT_FAST if contract == "fast" else abi.HS_CONTRACT_EXACT
    wl.contract = contract
    return wl


# ---- measurement helpers ----------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], 0.0, [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_median": float(np.median(power)) if power else None}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def profiled_value(workload, key):
    """A per-frame figure of the step from the committed ncu summary
    (`key: value` lines): DRAM bytes, warp instructions."""
    path = os.path.join(ROOT, "profiles", f"step_{workload}.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def issue_roofline(workload, frame_ms, clk, sms):
    """The bound the step actually meets: warp instructions issued per
    second against one per scheduler per cycle (4 schedulers per SM) at the
    median SM clock sampled during the timed region. The instruction count
    per frame comes from the committed ncu capture of the same kernels."""
    inst = profiled_value(workload, "warp_instructions_per_frame")
    mhz = clk.get("sm_mhz") if clk else None
    if inst is None or not mhz:
        return None
    peak = 4.0 * sms * mhz * 1e6
    achieved = inst / (frame_ms * 1e-3)
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "warp_instructions_per_frame": inst,
            "source": f"profiles/step_{workload}.md (smsp__inst_executed.sum)"}


def oracle_frame_all(wl, state, f, nthreads):
    """One frame of the whole workload on the CPU oracle (FP32)."""
    import oracle
    from barbu_gb300 import scenarios
    t = (f + 1) * DT
    for s, (p, v, rest) in zip(wl.specs, state):
        if isinstance(s, scenarios.SkinnedSpec):
            dq = oracle.matrix_to_dual_quat(s.rig.matrices(f + 1))
            tg = oracle.skin_targets(rest, s.bones, s.weights, dq, np.float32)
            oracle.frame(p, v, s.sim, DT, seed=int(s.strand.seed), spheres=s.spheres_at(f + 1), root_targets=tg,
                         nthreads=nthreads)
            continue
        wind = scenarios.wind_at(t) if s.wind else None
        m = s.transform(t)
        tg = oracle.rigid_targets(rest, m, np.float32) if m is not None else None
        oracle.frame(p, v, s.sim, DT, seed=int(s.strand.seed), wind=wind, spheres=s.spheres_at(t),
                     root_targets=tg, nthreads=nthreads)


def oracle_state(wl):
    import oracle
    out = []
    for s in wl.specs:
        p, v = oracle.init(s.roots, s.normals, s.strand, dtype=np.float32, lengths=s.lengths)
        out.append((p, v, p[:, 0, :3].copy()))
    return out


def cpu_oracle_rate(wl, seconds, nthreads, frames_max=300):
    state = oracle_state(wl)
    done, t0 = 0, time.perf_counter()
    while done < frames_max:
        oracle_frame_all(wl, state, done, nthreads)
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return wl.points_per_frame * done / el, done, el


def run_reference(args):
    """--impl reference: the oracle's FP32 restatement on the host cores."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    wl = make_workload(args.workload, args.strands)
    threads = oracle.max_threads()
    state = oracle_state(wl)
    steps = max(1, min(args.steps, 10))
    warm = min(args.warmup, 2)
    for f in range(warm):
        oracle_frame_all(wl, state, f, threads)
    t0 = time.perf_counter()
    for f in range(steps):
        oracle_frame_all(wl, state, warm + f, threads)
    el = time.perf_counter() - t0
    val = wl.points_per_frame * steps / el
    out = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": METRIC, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * el / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded groom generators)",
        "config": wl.config(args.gpus),
        "contract": CONTRACTS["exact"] + " (the host cannot run the GPU's rsqrt.approx)",
        "cpu_baseline": {"value": val, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"the whole {wl.name} workload, {steps} frames (oracle FP32 restatement of the "
                                   "reference step; the reference itself is a GLSL compute pass)"},
        "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def timed_frames(torch, ctx, stream, K, f0, do_frame, label="timed"):
    """K frames between two events on the library's stream; returns
    (elapsed ms, mean frame ms). No per-frame events: on the small groom a
    frame is ~25 us of device time, and per-frame event records would make
    the loop host-bound."""
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # The NVTX range lets a profiler select the timed launches (--nvtx-include timed/).
    torch.cuda.nvtx.range_push(label)
    with torch.cuda.stream(stream):
        t_start.record(stream)
        for k in range(K):
            do_frame(f0 + k)
        t_end.record(stream)
    torch.cuda.nvtx.range_pop()
    ctx.sync()
    torch.cuda.synchronize()
    el = t_start.elapsed_time(t_end)
    return el, el / K


def csrc_hash() -> str:
    """sha256 (first 16 hex digits) of the kernel sources, in name order: the
    committed ncu summaries record the hash they were captured at."""
    import hashlib
    d = os.path.join(ROOT, "barbu_gb300", "csrc")
    h = hashlib.sha256()
    for name in sorted(os.listdir(d)):
        if name.endswith((".cu", ".cuh", ".h")):
            h.update(name.encode())
            with open(os.path.join(d, name), "rb") as f:
                h.update(f.read())
    return h.hexdigest()[:16]


def profile_meta(workload):
    """(hash the profile was captured at, whether it matches the sources)."""
    path = os.path.join(ROOT, "profiles", f"step_{workload}.md")
    captured = None
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("csrc_hash:"):
                    captured = line.split(":", 1)[1].strip()
    except OSError:
        pass
    return captured, captured is not None and captured == csrc_hash()


def measure(args, torch, ctx, stream, wl, K, W, E, cpu_seconds, dist, world, rank, local, autotune=False):
    """One workload: device-timed frames (value), the plain per-groom path
    (batched only), end to end through the public API, the roofline and the
    CPU baseline. Returns the workload's JSON fields."""
    total_frames = W + 2 * K + 3 * (E2E_RUNS + 1) * E + 8
    wl.ctx = ctx
    wl.setup(ctx, total_frames)
    batched = isinstance(wl, Batched)
    tuned = 0
    if batched and autotune:
        wl.inputs(0)
        tuned = ctx.autotune(wl.grooms, DT)

    def frame(f):
        wl.inputs(f)
        wl.step(ctx)

    f = 0
    for _ in range(W):
        frame(f)
        f += 1
    ctx.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    n0 = ctx.launch_count()
    el_ms, frame_ms = timed_frames(torch, ctx, stream, K, f, frame)
    launches = ctx.launch_count() - n0
    f += K
    clk = clocks.stop()
    if dist:
        t = torch.tensor([el_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        el_ms = float(t.item())
        dist.barrier()
    value = world * wl.points_per_frame * K / (el_ms * 1e-3)

    plain = None
    if batched:
        for _ in range(3):
            wl.plain_step(f)
            f += 1
        ctx.sync()
        if dist:
            dist.barrier()
        pel_ms, pframe_ms = timed_frames(torch, ctx, stream, K, f, wl.plain_step, "timed_plain")
        f += K
        if dist:
            t = torch.tensor([pel_ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            pel_ms = float(t.item())
        pvalue = world * wl.points_per_frame * K / (pel_ms * 1e-3)
        plain = {"value": pvalue, "unit": METRIC, "ms_per_step": pel_ms / K,
                 "path": "one hs_update launch per groom per frame (64 launches)",
                 "batched_over_plain": value / pvalue}

    # End to end through the public API with host buffers, on the frames
    # that follow the timed region (the headline first: the skinned
    # workload's cost drifts with its animation). Pipelined: each frame's
    # readback is queued behind its update, then the previous frame's is
    # waited for (hs_readback_drain to 1), so frame f's copy to host (a
    # second stream) runs while frame f + 1 updates and is snapshotted; two
    # host buffers take turns; every frame's copy completes inside the
    # timed region. Headline: (x, y, z) per point (the rest lengths being
    # constant); then the same loop with (x, y, z, rest), and the blocking
    # hs_readback one frame at a time. Several grooms go through
    # hs_readback_many_async (one copy a frame). Each loop runs once
    # untimed, then is timed E2E_RUNS times and reports the median run: on
    # GB300 the first run of a loop was at times down to a sixth of the
    # next runs' rate, in a different loop from one process to the next.
    def pipelined(f, hosts, queue):
        ctx.sync()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(E):
            frame(f)
            queue(hosts[k % 2])
            ctx.readback_drain(1)
            f += 1
        ctx.readback_drain(0)
        return time.perf_counter() - t0, f

    hosts3 = [wl.host_buffers(torch, 3)[0] for _ in range(2)]
    d2h3 = sum(b.nbytes for b in hosts3[0])
    host, d2h = wl.host_buffers(torch)
    hosts4 = [host, wl.host_buffers(torch)[0]]
    # Untimed: the first readbacks create both staging buffers (at the
    # larger size first), the copy stream and its events, and make the first
    # copy into each host buffer (whose pages the copy engine maps at first
    # use).
    for h4 in hosts4:
        wl.readback_async(h4)
    ctx.readback_wait()
    for h3 in hosts3:
        wl.readback_xyz_async(h3)
    ctx.readback_wait()

    def blocking(f):
        ctx.sync()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(E):
            frame(f)
            wl.readback(host)
            f += 1
        return time.perf_counter() - t0, f

    def runs(f, loop):
        _, f = loop(f)  # untimed
        secs = []
        for _ in range(E2E_RUNS):
            s, f = loop(f)
            secs.append(s)
        return secs, f

    e2e_runs, f = runs(f, lambda f: pipelined(f, hosts3, wl.readback_xyz_async))
    del hosts3
    xyzw_runs, f = runs(f, lambda f: pipelined(f, hosts4, wl.readback_async))
    del hosts4
    sync_runs, f = runs(f, blocking)
    del host
    e2e_s, xyzw_s, sync_s = (sorted(r)[len(r) // 2] for r in (e2e_runs, xyzw_runs, sync_runs))
    if dist:
        t = torch.tensor([e2e_s, xyzw_s, sync_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s, xyzw_s, sync_s = (float(x) for x in t.tolist())
    e2e_value = world * wl.points_per_frame * E / e2e_s
    e2e_xyzw_value = world * wl.points_per_frame * E / xyzw_s
    e2e_sync_value = world * wl.points_per_frame * E / sync_s

    def run_values(secs):
        return [world * wl.points_per_frame * E / x for x in secs]

    export = None
    if not batched and rank == 0:
        # Device-to-device export of the positions in the renderer's order.
        from barbu_gb300 import abi
        g = wl.g
        buf = torch.empty(4 * wl.points, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for _ in range(3):
            g.export(buf.data_ptr(), buf.numel(), abi.HS_EXPORT_STRAND_MAJOR)
        ems, _ = timed_frames(torch, ctx, stream, 20, 0,
                              lambda f: g.export(buf.data_ptr(), buf.numel(), abi.HS_EXPORT_STRAND_MAJOR),
                              "timed_export")
        per = ems / 20
        export = {"layout": "strand-major positions", "bytes_moved": 2 * 16 * wl.points, "ms": per,
                  "gbs": 2 * 16 * wl.points / (per * 1e-3) / 1e9}
        del buf
    peak, peak_kind = measured_hbm_peak()
    alg_bytes = BYTES_PER_POINT * wl.points
    achieved = alg_bytes / (frame_ms * 1e-3) / 1e9
    prof = wl.name + ("_fast" if wl.contract == "fast" else "")  # the workload's profile summary
    traffic = profiled_value(prof, "traffic_bytes_per_frame")
    prof_hash, prof_current = profile_meta(prof)
    issue = issue_roofline(prof, frame_ms, clk, torch.cuda.get_device_properties(0).multi_processor_count)
    if issue is not None:
        issue["stale"] = not prof_current

    cpu = None
    if rank == 0 and world == 1 and cpu_seconds > 0:
        import oracle
        thr = oracle.max_threads()
        rate, frames, secs = cpu_oracle_rate(wl, cpu_seconds, thr)
        cpu = {"value": rate, "unit": METRIC, "cores": thr, "kind": "port",
               "sample": f"the whole {wl.name} workload for {frames} frames ({secs:.1f} s), oracle FP32, OpenMP"}
    wl.destroy()

    if batched:
        kernel = "k_step_batch_stream_tmem (all buckets, one graph per frame)"
    else:
        if getattr(wl, "mapping", "").startswith("lane"):
            kernel = "k_step_lanes"
        else:
            kernel = "k_step_stream_tmem" if wl.specs[0].npoints > 8 else "k_step (registers)"
    out = {
        "value": value, "unit": METRIC, "ms_per_step": el_ms / K, "steps": K, "warmup": W,
        "config": wl.config(world),
        "contract": CONTRACTS[wl.contract],
        **({"mapping": wl.mapping} if hasattr(wl, "mapping") else {}),
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": wl.h2d_bytes(),
                "d2h_bytes_per_step": d2h3, "steps": E,
                "runs": run_values(e2e_runs), "statistic": f"median of {E2E_RUNS} timed runs of {E} steps, after one untimed run",
                "path": "update + asynchronous readback per frame of (x, y, z) of every point "
                        "(hs_readback_many_async for several grooms, hs_readback_xyz_async for one), "
                        "copy of frame f overlapping the update and snapshot of frame f+1",
                "xyzw": {"value": e2e_xyzw_value, "d2h_bytes_per_step": d2h, "runs": run_values(xyzw_runs),
                         "path": "update + asynchronous readback per frame of (x, y, z, rest), pipelined"},
                "synchronous": {"value": e2e_sync_value, "d2h_bytes_per_step": d2h, "runs": run_values(sync_runs),
                                "path": "update + hs_readback (blocking) per frame"}},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic if prof_current else None,
                     "traffic_profiled": traffic, "profile_csrc_hash": prof_hash,
                     "csrc_hash": csrc_hash(), "profile_stale": not prof_current,
                     "peak_source": peak_kind, "kernel": kernel, "frame_ms": frame_ms,
                     "algorithmic_bytes_per_frame": alg_bytes, "issue": issue},
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    if plain is not None:
        out["plain"] = plain
        out["autotune_trials"] = tuned
    if export is not None:
        out["export"] = export
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from barbu_gb300 import hairsim

    wl = make_workload(args.workload, args.strands, args.contract)
    ctx = hairsim.Context()
    stream = torch.cuda.ExternalStream(ctx.stream)
    K, W, E = args.steps, args.warmup, args.e2e_steps
    cpu_s = 0.0 if args.no_cpu_baseline else args.cpu_seconds
    batched = isinstance(wl, Batched)
    res = measure(args, torch, ctx, stream, wl, K, W, E, cpu_s, dist, world, rank, local,
                  autotune=batched and not args.no_autotune)

    # The batched workload again under the other contract (EXACT beside a
    # FAST line: the arithmetic the FP32 oracle reproduces bit for bit),
    # with its own per-groom path for the batched-over-plain ratio.
    alt_name = "exact" if args.contract == "fast" else "fast"
    alt = None
    if batched and not args.no_alt_contract:
        alt = measure(args, torch, ctx, stream, make_workload("batched", None, alt_name), K, W, min(E, 10), 0.0,
                      dist, world, rank, local, autotune=not args.no_autotune)
        alt = {k: alt[k] for k in ("value", "unit", "ms_per_step", "contract", "e2e", "gpu_launches", "roofline",
                                   "plain", "clocks") if k in alt}

    # The default line also carries the single-groom configurations (their
    # own device-timed value, roofline, end-to-end figure and a shorter CPU
    # sample), so that every configuration is measured in the same run.
    others = {}
    if batched and not args.no_others:
        for name, k, e, c in (("plain", K, min(E, 10), min(cpu_s, 5.0)), ("large", K, min(E, 5), min(cpu_s, 5.0)),
                              ("skinned", max(3, K // 2), min(E, 3), min(cpu_s, 8.0))):
            others[name] = measure(args, torch, ctx, stream, make_workload(name, None, args.contract), k, W, e, c,
                                   dist, world, rank, local)

    served = None
    if batched and not args.no_served:
        from barbu_gb300 import abi
        code = {"fast": abi.HS_CONTRACT_FAST, "exact": abi.HS_CONTRACT_EXACT}
        budget = int(args.served_budget_gb * (1 << 30))
        shapes = ServedShapes(contract=code[args.contract])
        served = {"budget_bytes": budget, "substeps": 4, "points_per_strand": [8, 16, 24, 32],
                  "contract": CONTRACTS[args.contract],
                  "sizes": "the batched workload's distribution: strands log-uniform in [1024, 131072], "
                           "points per strand from {8, 16, 24, 32}, 1-16 spheres; lifetimes U[30, 300] frames",
                  "streams": [run_served(ctx, shapes, r, args.served_ticks, 60, budget) for r in (20, 100, 500)],
                  "resident_64": run_fixed(ctx, shapes, 64, args.served_ticks, 10, budget)}
        # The other reading of "the config-2 size distribution": the large
        # groom's kind, 32 points per strand, 4,096 to 262,144 strands.
        large = ServedShapes(lo=4096, hi=262144, points=(32,), seed=0xBA5B0 + 6, contract=code[args.contract])
        served["resident_64_large"] = dict(run_fixed(ctx, large, 64, args.served_ticks, 10, budget),
                                           sizes="strands log-uniform in [4096, 262144], 32 points per strand")
        large_alt = ServedShapes(lo=4096, hi=262144, points=(32,), seed=0xBA5B0 + 6, contract=code[alt_name])
        served[f"resident_64_large_{alt_name}"] = dict(
            run_fixed(ctx, large_alt, 64, args.served_ticks, 10, budget),
            sizes=f"as resident_64_large, every groom under the {alt_name.upper()} contract")
    tune_choices = ctx.tune_entries()
    tess = run_tess(torch, ctx, stream) if (rank == 0 and not args.no_tess) else None
    ctx.close()
    if rank == 0:
        out = {"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded groom generators; the reference has no dataset)"}
        out.update({k: v for k, v in res.items() if k not in ("value", "ms_per_step", "steps", "warmup")})
        if batched:
            out["autotune_choices"] = tune_choices
        if others:
            out["workloads"] = others
        if alt is not None:
            out[f"{alt_name}_contract"] = alt
        if served is not None:
            out["served"] = served
        if tess is not None:
            out["tess"] = tess
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
