"""Uneven batches (msl_run_jobs): jobs of different grids, thicknesses, energies and
illumination advanced in lockstep equal the job-by-job slice loop and the oracle."""
import numpy as np
import pytest

from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def _jobs(seed=5, n=10):
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n):
        side = int(rng.choice([64, 128, 256]))
        ax = float(rng.uniform(8.0, 20.0))
        by = ax * float(rng.uniform(0.9, 1.1))
        nt = int(rng.integers(1, 4))
        nslice = int(rng.integers(2, 12))
        kev = float(rng.choice([80.0, 200.0, 300.0]))
        V = np.zeros((nt, side, side))
        for l in range(nt):
            ix = rng.integers(0, side, 8)
            iy = rng.integers(0, side, 8)
            V[l, ix, iy] = rng.uniform(50, 400, 8)
        t = O.transmission(V, kev, ax, by, np.complex64)
        d = dict(trans=t, ax=ax, by=by, kev=kev, dz=rng.uniform(1.0, 2.0, nt),
                 layer_seq=rng.integers(0, nt, nslice))
        if j % 3 == 1:
            d["probe"] = (float(rng.uniform(0.4, 1.2)), float(rng.uniform(0, ax)), float(rng.uniform(0, by)))
        jobs.append(d)
    return jobs


def test_uneven_batch_matches_oracle_and_single_runs(ctx):
    jobs = _jobs()
    outs = ctx.run_jobs(jobs)
    for d, w in zip(jobs, outs):
        nt, nx, ny = d["trans"].shape
        mask = O.band_mask(nx, ny, d["ax"], d["by"])
        props = [O.propagator_tables(nx, ny, d["ax"], d["by"], d["kev"], dz, precision="f64") for dz in d["dz"]]
        if "probe" in d:
            k_ap, x, y = d["probe"]
            psi0 = O.probe(nx, ny, d["ax"], d["by"], d["kev"], 0.0, k_ap, 0.0, 0.0, [[x, y]], np.complex128)[0]
        else:
            psi0 = np.ones((nx, ny), np.complex128)
            single = ctx.multislice(d["trans"], d["dz"], d["layer_seq"], d["ax"], d["by"], d["kev"])[0]
            assert np.array_equal(single, w)
        ref, _ = O.multislice(psi0, d["trans"].astype(np.complex128), props, d["layer_seq"], mask)
        assert O.rel_l2(w, ref) < 2e-5


def test_uneven_batch_rejects_bad_job(ctx):
    from multislice_gb300 import MslError
    jobs = _jobs(n=3)
    jobs[1]["layer_seq"] = np.array([0, 7])
    with pytest.raises(MslError) as e:
        ctx.run_jobs(jobs)
    assert "job" in str(e.value)


def test_uneven_workload_every_side(ctx):
    """The uneven-batch workload at reduced thickness: amorphous specimens on every
    grid side 256-1024, 80-300 kV, plane waves and probes mixed, built on the GPU
    and run in one lockstep loop; each job equals its own run, the smallest also
    the FP64 oracle."""
    from multislice_gb300 import specimen as S
    descs = S.uneven_jobs(3, 10, max_slices=26, max_box=32.0)
    assert sorted({d["n"] for d in descs}) == [256, 384, 512, 768, 1024]
    jobs = []
    for d in descs:
        s, n = d["spec"], d["n"]
        v = ctx.potential(s, n, n, d["nslice"], 3.0)
        t = ctx.transmission(v, s.ax, s.by, d["kev"])
        job = dict(trans=t, ax=s.ax, by=s.by, kev=d["kev"], dz=d["dz"], layer_seq=np.arange(d["nslice"]))
        if d["probe"] is not None:
            job["probe"] = d["probe"]
        jobs.append(job)
    outs = ctx.run_jobs(jobs)
    for job, w in zip(jobs, outs):
        if "probe" in job:
            alone = ctx.run_jobs([job])[0]
            assert O.rel_l2(w, alone) < 1e-6
        else:
            alone = ctx.multislice(job["trans"], job["dz"], job["layer_seq"], job["ax"], job["by"], job["kev"])[0]
            assert np.array_equal(w, alone)
        assert np.isfinite(w).all()
    j = min(range(len(jobs)), key=lambda i: descs[i]["n"] * descs[i]["nslice"])
    job = jobs[j]
    nt, nx, ny = job["trans"].shape
    props = [O.propagator_tables(nx, ny, job["ax"], job["by"], job["kev"], job["dz"], precision="f64")] * nt
    if "probe" in job:
        k_ap, x, y = job["probe"]
        psi0 = O.probe(nx, ny, job["ax"], job["by"], job["kev"], 0.0, k_ap, 0.0, 0.0, [[x, y]], np.complex128)[0]
    else:
        psi0 = np.ones((nx, ny), np.complex128)
    ref, _ = O.multislice(psi0, job["trans"].astype(np.complex128), props, job["layer_seq"],
                          O.band_mask(nx, ny, job["ax"], job["by"]))
    assert O.rel_l2(outs[j], ref) < 2e-5


def test_uneven_batch_same_under_memory_cap():
    """Groups run concurrently on their own streams without a memory cap and one
    after another in shared buffers under one; the exit waves are identical."""
    from multislice_gb300 import Context
    jobs = _jobs(seed=9, n=12)
    with Context(0) as c:
        free = c.run_jobs(jobs)
        c.set_memory_limit(1 << 30)
        capped = c.run_jobs(jobs)
        assert c.memory_in_use() <= 1 << 30
    for a, b in zip(free, capped):
        assert np.array_equal(a, b)
