"""Multi-rank host logic on CPU: two gloo ranks shard a STEM raster, each runs its
block, one gather assembles the image, which equals the single-rank result."""
import os
import socket

import numpy as np
import pytest

from multislice_gb300.sharding import probe_shard

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _small_stem_problem():
    from oracle import msl_oracle as O
    rng = np.random.default_rng(11)
    n, a, kev = 64, 12.0, 200.0
    V = np.zeros((2, n, n))
    for l in range(2):
        for _ in range(6):
            x, y = rng.random(2) * a
            ix, iy = int(x / a * n), int(y / a * n)
            V[l, ix, iy] += 400.0
    T = O.transmission(V, kev, a, a, np.complex128)
    props = [O.propagator_tables(n, n, a, a, kev, 2.0, precision="f64")] * 2
    mask = O.band_mask(n, n, a, a)
    xy = np.stack(np.meshgrid(np.arange(5) * 2.3, np.arange(3) * 3.1, indexing="ij"), -1).reshape(-1, 2)
    dm = O.detector_masks(n, n, a, a, [(0.0, 1.0), (1.0, 3.0)])
    return T, props, mask, xy, dm, kev, a, n


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from oracle import msl_oracle as O
    from multislice_gb300.sharding import gather_detector_sums

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    T, props, mask, xy, dm, kev, a, n = _small_stem_problem()
    lo, hi = probe_shard(len(xy), rank, world)
    P = O.probe(n, n, a, a, kev, 0.0, 0.8, 0.0, 0.0, xy[lo:hi], np.complex128)
    local = O.stem(T, props, [0, 1, 0, 1], mask, P, dm, [3])
    full = gather_detector_sums(local, len(xy))
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_probe_shard_covers_everything_once():
    for n in (1, 7, 4096):
        for w in (1, 2, 3, 8):
            spans = [probe_shard(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
                assert a1 == b0
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_match_single_rank(tmp_path):
    import torch.multiprocessing as mp
    from oracle import msl_oracle as O

    out = str(tmp_path / "full.npy")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    full = np.load(out)
    T, props, mask, xy, dm, kev, a, n = _small_stem_problem()
    P = O.probe(n, n, a, a, kev, 0.0, 0.8, 0.0, 0.0, xy, np.complex128)
    ref = O.stem(T, props, [0, 1, 0, 1], mask, P, dm, [3])
    np.testing.assert_allclose(full, ref, rtol=1e-12, atol=1e-12)


def test_job_shard_covers_every_job_once_and_balances():

    from multislice_gb300.sharding import job_cost, job_shard
    rng = np.random.default_rng(0)
    sides = rng.choice([256, 384, 512, 768, 1024], 256)
    slices = rng.integers(20, 301, 256)
    costs = [job_cost(n, s) for n, s in zip(sides, slices)]
    for world in (1, 2, 4, 8):
        parts = [job_shard(costs, r, world) for r in range(world)]
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(256))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs)      # greedy bound
        assert max(loads) / (sum(costs) / world) < 1.05            # near even at 256 jobs

