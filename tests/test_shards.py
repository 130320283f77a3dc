"""A groom split across two processes (gloo, CPU) reproduces the whole.

Each rank simulates its contiguous strand range with strand_base set, the
positions are gathered on the host, and rank 0 compares them bit for bit
with the unsplit groom. The compute here is the oracle (no GPU in this
test); what is under test is the partition, the strand_base bookkeeping and
the gather that a multi-GPU run uses.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    import torch.distributed as dist

    import oracle
    from barbu_gb300 import scenarios, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        spec = scenarios.large(ns=1001, npoints=8, nspheres=6)
        lo, hi = shard.shard_range(spec.nstrands, rank, world)
        sp = shard.shard_params(spec.strand, lo)
        p, v = oracle.init(spec.roots[lo:hi], spec.normals[lo:hi], sp, dtype=np.float32, lengths=spec.lengths[lo:hi])
        for f in range(4):
            w = scenarios.wind_at((f + 1) / 60)
            oracle.frame(p, v, spec.sim, 1 / 60, seed=int(sp.seed), wind=w, spheres=spec.spheres, strand_base=lo,
                         nthreads=1)
        whole = shard.gather(p, spec.nstrands, world, dist)
        if rank == 0:
            q.put(whole)
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_match_unsplit_groom():
    import torch.multiprocessing as mp

    import oracle
    from barbu_gb300 import scenarios
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    spec = scenarios.large(ns=1001, npoints=8, nspheres=6)
    p, v = oracle.init(spec.roots, spec.normals, spec.strand, dtype=np.float32, lengths=spec.lengths)
    for f in range(4):
        w = scenarios.wind_at((f + 1) / 60)
        oracle.frame(p, v, spec.sim, 1 / 60, seed=int(spec.strand.seed), wind=w, spheres=spec.spheres)
    np.testing.assert_array_equal(got.view(np.uint32), p.view(np.uint32))


@pytest.mark.parametrize("n,world", [(10, 3), (1001, 2), (5, 8), (0, 2)])
def test_shard_ranges_cover_exactly(n, world):
    from barbu_gb300 import shard
    ranges = [shard.shard_range(n, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    for (a, b), (c, d) in zip(ranges, ranges[1:]):
        assert b == c and b >= a
    sizes = [b - a for a, b in ranges]
    assert max(sizes) - min(sizes) <= 1
