"""Benchmark of the hair-strand simulation step on GB300.

Metric: strand-point substeps/s = strands x points x substeps x frames / s.
A step is one frame: every strand of the workload advanced by S substeps.

Workloads (seeded synthetic grooms, barbu_gb300/scenarios.py):
  large  262,144 strands x 32 points, 16 spheres, wind, 8 substeps (default)
  plain  4,096 strands x 16 points, 1 moving sphere, 4 substeps

Our arm (default): the CUDA library through its C-ABI.
  value     device-timed: K frames back to back with the state resident in
            HBM (its 268 MB exceed the 129 MB L2, so no flush is needed),
            CUDA events on the library's stream, max over ranks.
  e2e       the same frames through the public API with host buffers: per
            frame the per-frame inputs (wind, spheres, root transform) go in
            from host memory and the positions the renderer consumes come
            back to pinned host memory.
  roofline  the step kernel against measured HBM bandwidth: algorithmic
            bytes = 64 B per control point per frame (float4 position and
            velocity, read once and written once).
  cpu_baseline  the oracle's FP32 instantiation, OpenMP over all host
            cores, on the same workload for about 10 s (rank 0, N = 1).
--impl reference: the oracle's FP32 instantiation (the reference path is a
GLSL compute shader with no CPU implementation and no graphics stack on
this machine; the oracle is its C++ restatement) timed on the host cores.

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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["large", "plain"], default="large")
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def make_spec(name):
    from barbu_gb300 import scenarios
    return scenarios.large() if name == "large" else scenarios.plain()


def frame_inputs(spec, f, dt):
    from barbu_gb300 import scenarios
    t = (f + 1) * dt
    wind = scenarios.wind_at(t) if spec.wind else None
    return wind, spec.transform(t), spec.spheres_at(t)


def config_of(spec, name, args, world):
    return {
        "workload": name,
        "strands": spec.nstrands,
        "points_per_strand": spec.npoints,
        "substeps": int(spec.sim.substeps),
        "spheres": int(spec.spheres.shape[0]),
        "mode": "dftl",
        "dt": 1.0 / 60.0,
        "replicas": world,
        "l2": "state (64 B/point) larger than the 129 MB L2; no flush",
    }


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
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def profiled_traffic(workload):
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"step_kernel_{workload}.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def cpu_oracle_rate(spec, seconds, nthreads=0, frames_max=300):
    """FP32 oracle over the full workload, frames until ~seconds elapse."""
    import oracle
    from barbu_gb300 import abi  # noqa: F401
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float32, lengths=spec.lengths)
    rest = p[:, 0, :3].copy()
    dt = 1.0 / 60.0
    pts = spec.nstrands * spec.npoints * int(spec.sim.substeps)
    done, t0 = 0, time.perf_counter()
    while done < frames_max:
        wind, m, sph = frame_inputs(spec, done, dt)
        tg = oracle.rigid_targets(rest, m, np.float32) if m is not None else None
        oracle.frame(p, v, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=sph, root_targets=tg,
                     nthreads=nthreads)
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return pts * done / el, done, el


def run_reference(args, name):
    """--impl reference: the oracle's FP32 restatement on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    spec = make_spec(name)
    threads = oracle.max_threads()
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float32, lengths=spec.lengths)
    rest = p[:, 0, :3].copy()
    dt = 1.0 / 60.0

    def step(f):
        wind, m, sph = frame_inputs(spec, f, dt)
        tg = oracle.rigid_targets(rest, m, np.float32) if m is not None else None
        oracle.frame(p, v, spec.sim, dt, seed=int(spec.strand.seed), wind=wind, spheres=sph, root_targets=tg,
                     nthreads=threads)

    steps = min(args.steps, 20)
    warm = min(args.warmup, 3)
    for f in range(warm):
        step(f)
    t0 = time.perf_counter()
    for f in range(steps):
        step(warm + f)
    el = time.perf_counter() - t0
    pts = spec.nstrands * spec.npoints * int(spec.sim.substeps)
    val = pts * steps / el
    unit = "strand-point substeps/s"
    out = {
        "impl": "reference",
        "metric": "strand-point substeps/s",
        "value": val,
        "unit": unit,
        "n_gpus": args.gpus,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded groom generators)",
        "config": config_of(spec, name, args, 1),
        "cpu_baseline": {"value": val, "unit": unit, "cores": threads, "kind": "port",
                         "sample": f"full {name} groom, {steps} frames (oracle FP32 restatement of the "
                                   "reference shader; the reference itself is a GLSL compute pass)"},
        "e2e": {"value": val, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    args = parse()
    name = args.workload
    if args.impl == "reference":
        run_reference(args, name)
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

    spec = make_spec(name)
    ctx = hairsim.Context()
    stream = torch.cuda.ExternalStream(ctx.stream)
    g = ctx.groom(spec.roots, spec.normals, spec.strand, spec.sim, lengths=spec.lengths)
    dt = 1.0 / 60.0
    f = 0

    def set_inputs(fi):
        wind, m, sph = frame_inputs(spec, fi, dt)
        if wind is not None:
            g.set_wind(wind)
        if m is not None:
            g.set_root_transform(m)
        g.set_spheres(sph)

    for _ in range(args.warmup):
        set_inputs(f)
        g.update(dt)
        f += 1
    ctx.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    n0 = ctx.launch_count()
    with torch.cuda.stream(stream):
        t_start.record(stream)
        for k in range(K):
            set_inputs(f)
            ev[k][0].record(stream)
            g.update(dt)
            ev[k][1].record(stream)
            f += 1
        t_end.record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    launches = ctx.launch_count() - n0
    clk = clocks.stop()
    el_ms = t_start.elapsed_time(t_end)
    kern_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    if dist:
        t = torch.tensor([el_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        el_ms = float(t.item())
        dist.barrier()

    pts_per_frame = spec.nstrands * spec.npoints * int(spec.sim.substeps)
    value = world * pts_per_frame * K / (el_ms * 1e-3)

    # End to end through the public API with host buffers.
    E = args.e2e_steps
    host_pos = torch.empty((spec.nstrands, spec.npoints, 4), dtype=torch.float32, pin_memory=True)
    host_np = host_pos.numpy()
    h2d = 4 * (3 + 16 + 4 * spec.spheres.shape[0])
    ctx.sync()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(E):
        set_inputs(f)
        g.update(dt)
        g.readback(host_np)
        f += 1
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * pts_per_frame * E / e2e_s
    d2h = host_np.nbytes

    peak, peak_kind = measured_hbm_peak()
    alg_bytes = BYTES_PER_POINT * spec.nstrands * spec.npoints
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    traffic = profiled_traffic(name)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        thr = oracle.max_threads()
        rate, frames, secs = cpu_oracle_rate(spec, args.cpu_seconds, nthreads=thr)
        cpu = {"value": rate, "unit": "strand-point substeps/s", "cores": thr, "kind": "port",
               "sample": f"full {name} groom for {frames} frames ({secs:.1f} s), oracle FP32, OpenMP"}

    g.destroy()
    ctx.close()
    if rank == 0:
        out = {
            "metric": "strand-point substeps/s",
            "value": value,
            "unit": "strand-point substeps/s",
            "n_gpus": world,
            "steps": K,
            "warmup": args.warmup,
            "ms_per_step": el_ms / K,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded groom generators; the reference has no dataset)",
            "config": config_of(spec, name, args, world),
            "e2e": {"value": e2e_value, "unit": "strand-point substeps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": E},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "k_step (plain per-groom)", "kernel_ms": kern_ms,
                         "algorithmic_bytes_per_launch": alg_bytes},
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
