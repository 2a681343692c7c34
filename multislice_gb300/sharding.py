"""Probe sharding across ranks (one process per GPU).

STEM probes (and frozen-phonon configurations) are independent: the reference
runs them in a serial loop (MSProjectReuse.cs:254-347, MSProjectUseOnce.cs:235-273).
Across GPUs each rank takes a contiguous block of the probe list, runs the whole
slice loop for its block with no communication, and one gather of the detector
sums at the end assembles the image.  There is no per-slice exchange.
"""
from __future__ import annotations

import numpy as np


def probe_shard(nprobe, rank, world):
    """[lo, hi) of the probes rank `rank` of `world` owns (contiguous, sizes differ by <= 1)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(nprobe), int(world))
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def gather_detector_sums(local, nprobe, group=None):
    """All-gather per-rank detector blocks [n_local, ...] into the full [nprobe, ...] array.

    Uses torch.distributed (gloo on CPU, nccl on GPUs); returns a numpy array on
    every rank."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    local = np.ascontiguousarray(local, dtype=np.float64)
    tail = local.shape[1:]
    width = -(-int(nprobe) // world)
    buf = np.zeros((width,) + tail, np.float64)
    buf[: len(local)] = local
    t = torch.from_numpy(buf)
    backend = dist.get_backend(group)
    if backend == "nccl":
        t = t.cuda()
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    out = []
    for r, p in enumerate(parts):
        lo, hi = probe_shard(nprobe, r, world)
        out.append(p.cpu().numpy()[: hi - lo])
    return np.concatenate(out, axis=0)
