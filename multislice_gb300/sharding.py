"""Probe and job sharding across ranks (one process per GPU).

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


def job_cost(n, nslice):
    """Relative cost of one job of the uneven batch: two passes of N log N line
    transforms over N lines per slice."""
    return float(n) * float(n) * np.log2(float(n)) * float(nslice)


def job_shard(costs, rank, world):
    """Indices of the jobs rank `rank` of `world` runs: jobs of very different
    sizes and thicknesses are dealt largest first to the least-loaded rank (the
    same on every rank, so no communication is needed).  Each rank then runs its
    jobs as one uneven batch (msl_run_jobs)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    costs = np.asarray(costs, dtype=np.float64)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    owner = np.empty(len(costs), dtype=np.int64)
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += costs[i]
    return np.nonzero(owner == rank)[0]


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
