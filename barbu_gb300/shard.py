"""Splitting a groom across processes (one GPU each).

Strands are independent, so a groom shards into contiguous strand ranges
with no exchange during the step. `strand_base` keeps each strand's hashed
draws (length and wind jitter) those of the whole groom, so the shards
reproduce the unsplit groom bit for bit. Only outputs are gathered, on the
host side, when a caller wants the whole groom in one place.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def shard_range(nstrands: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced strand range [lo, hi) of `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    base, extra = divmod(nstrands, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_params(sp: abi.StrandParams, lo: int) -> abi.StrandParams:
    """Strand parameters of the shard starting at strand `lo`."""
    out = abi.StrandParams()
    C.memmove(C.byref(out), C.byref(sp), C.sizeof(abi.StrandParams))
    out.strand_base = int(sp.strand_base) + lo
    return out


def gather(local: np.ndarray, nstrands: int, world: int, dist) -> np.ndarray:
    """All-gathers per-rank strand-major arrays (ns_r, N, 4) into the whole
    groom on every rank (host-side aggregation through torch.distributed)."""
    import torch
    n, four = local.shape[1], local.shape[2]
    width = max(shard_range(nstrands, r, world)[1] - shard_range(nstrands, r, world)[0] for r in range(world))
    pad = np.zeros((width, n, four), dtype=local.dtype)
    pad[: local.shape[0]] = local
    parts = [torch.zeros_like(torch.from_numpy(pad)) for _ in range(world)]
    dist.all_gather(parts, torch.from_numpy(pad))
    out = []
    for r in range(world):
        lo, hi = shard_range(nstrands, r, world)
        out.append(parts[r].numpy()[: hi - lo])
    return np.concatenate(out)
