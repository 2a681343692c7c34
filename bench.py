"""Benchmark: STEM probe-slices/s on the SrTiO3 512^2, 4096-probe HAADF/ABF scan.

Workload (one step): SrTiO3 [001], 8x8x50 cells, 512x512 grid over 31.24 A,
100 slices of 1.9525 A, 200 kV, 25 mrad aberration-free probe, 64x64 raster
over the central 2x2 cells (4096 probes), HAADF 80-200 mrad and ABF 11-22 mrad
detector sums after the last slice.  Synthetic specimen on ideal sites.

  value : msl_stem_scan over all 4096 probes with the transmission functions
          already resident in HBM (device buffers in and out).
  e2e   : the whole user call chain from host memory, copies included:
          msl_potential_build (host atoms) -> msl_transmission_build ->
          msl_stem_scan -> detector sums back in host memory.

--impl reference times the reference's CPU path (the oracle port of Kirkland's
mulslice loop with the C# probe and detector, scipy FFTs on all host threads)
on a bounded sample of the same workload.
"""
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

METRIC = "STEM probe-slices/s at 512^2 (SrTiO3, 4096-probe HAADF/ABF scan)"
UNIT = "probe-slices/s"
NSLICE = 100
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def workload():
    from multislice_gb300 import specimen as S
    cfg = S.config_srtio3_stem()
    return cfg


def peaks():
    try:
        with open(PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ our arm
def run_ours(args):
    import torch
    import torch.distributed as dist
    from multislice_gb300 import Context

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg = workload()
    spec = cfg["spec"]
    nx = ny = 512
    # weak scaling: every rank scans its own 4096-probe raster (shifted by one
    # probe step per rank so ranks never repeat work)
    xy = cfg["probe_xy"][: args.probes].copy()
    xy[:, 0] += rank * (2 * 3.905 / 64) / max(world, 1)
    nprobe = len(xy)
    dz = spec.cz / NSLICE
    seq = np.arange(NSLICE, dtype=np.int32)
    det_k = cfg["det_k"]

    ctx = Context(local)
    if args.batch:
        ctx.set_probe_batch(args.batch)
    if args.tc:
        ctx.set_schedule(nx, 3, 3)  # profiling aid: the tensor-core passes for the timed scan
    # device-resident inputs for `value`
    v_dev = torch.empty((NSLICE, nx, ny), dtype=torch.float32, device=dev)
    ctx.potential(spec, nx, ny, NSLICE, cfg["radius"], out=v_dev)
    t_dev = torch.empty((NSLICE, nx, ny, 2), dtype=torch.float32, device=dev)
    ctx.transmission(v_dev, spec.ax, spec.by, 200.0, out=t_dev)
    out_dev = torch.empty((nprobe, 1, len(det_k)), dtype=torch.float64, device=dev)

    def step():
        ctx.stem_scan(t_dev, dz, seq, spec.ax, spec.by, 200.0, cfg["k_ap"], xy, det_k, out=out_dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    l0 = ctx.launches
    ctx.profile(True)
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        barrier()
        t1 = time.perf_counter()
    prof = ctx.profile_read()
    ctx.profile(False)
    launches = ctx.launches - l0
    elapsed = t1 - t0
    if world > 1:
        tt = torch.tensor([elapsed], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        elapsed = float(tt.item())
    units = nprobe * NSLICE * world * args.steps
    value = units / elapsed

    # e2e: host atoms in, host detector sums out, through the public API
    res_host = np.empty((nprobe, 1, len(det_k)), np.float64)

    def e2e_step():
        ctx.potential(spec, nx, ny, NSLICE, cfg["radius"], out=v_dev)
        ctx.transmission(v_dev, spec.ax, spec.by, 200.0, out=t_dev)
        ctx.stem_scan(t_dev, dz, seq, spec.ax, spec.by, 200.0, cfg["k_ap"], xy, det_k, out=res_host)

    e_el = float("nan")
    if not args.no_e2e:
        e2e_step()
        barrier()
        e0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        barrier()
        e_el = time.perf_counter() - e0
    if world > 1:
        tt = torch.tensor([e_el], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e_el = float(tt.item())
    e2e_value = units / e_el if e_el == e_el else None   # None (JSON null) with --no-e2e
    h2d = spec.natom * (3 * 8 + 4) + 104 * 12 * 8 + nprobe * 2 * 8
    d2h = res_host.nbytes

    # roofline of the dominant kernel (the pass with the larger device time; the other beside it)
    hbm, peak_kind = peaks()
    rows = {}
    for kind in ("row", "col"):
        n, ms = prof[kind]
        per_launch = ms / max(n, 1)
        # algorithmic bytes per launch: every launch streams the batch's waves
        # once in and once out: 16 * nx * ny bytes per probe
        bytes_per_launch = 16.0 * nx * ny * nprobe
        rows[kind] = dict(launches=n, ms_per_launch=per_launch,
                          achieved_gbs=bytes_per_launch / (per_launch * 1e-3) / 1e9 if n else None)
    dom = "col" if prof["col"][1] >= prof["row"][1] else "row"
    ach = rows[dom]["achieved_gbs"]
    traffic = None
    tr_file = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tr_file):
        try:
            traffic = json.load(open(tr_file)).get(f"{dom}_pass_bytes_per_launch_4096")
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64/f32",
        "data": "synthetic (SrTiO3 on ideal sites, seeded raster)",
        "config": {"workload": "SrTiO3 [001] 8x8x50 cells, 512x512, 100 slices, 200 kV, "
                               "25 mrad probe, 64x64 raster (4096 probes), HAADF 80-200 + ABF 11-22 mrad",
                   "probes_per_gpu": nprobe, "slices": NSLICE, "grid": [nx, ny],
                   "l2": "inputs larger than L2 (waves 8.6 GB, transmission 210 MB)",
                   "parallelism": f"replicas x{world} (probe rasters per GPU)"},
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "chain": "potential_build(host atoms) + transmission_build + stem_scan(host out)"},
        "roofline": {"bound": "hbm", "kernel": f"{dom}_pass", "achieved": ach, "peak": hbm,
                     "unit": "GB/s", "frac": (ach / hbm) if ach else None, "traffic": traffic,
                     "peak_source": peak_kind, "passes": rows},
    }
    if rank == 0:
        if world == 1 and not args.no_cpu:
            full = out_dev.cpu().numpy()
            chk = full[: args.cpu_probes] if nprobe >= args.cpu_probes else None
            cb = cpu_baseline(cfg, args.cpu_probes, check=chk)
            acc = cb.pop("accuracy", None) or {}
            ref64 = None
            if not args.no_fp64:
                a64, ref64 = accuracy_fp64(cfg, xy, full, local)
                acc.update(a64)
            line["cpu_baseline"] = cb
            if acc:
                line["accuracy"] = acc
            if not args.no_variants:
                line["variants"] = run_variants(ctx, cfg, xy, full, ref64, args, t_dev)
        line["clocks"] = clk.summary()
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------- CPU baseline
def cpu_prepare(cfg):
    """Inputs of the CPU leg (not timed): the oracle's potential, transmission
    functions, propagator, band limit and detector masks of the workload."""
    from oracle import msl_oracle as O
    spec = cfg["spec"]
    nx = ny = 512
    fp = np.load(os.path.join(ROOT, "multislice_gb300", "data", "fparams.npy"))
    V = O.potential(spec.x, spec.y, spec.z, spec.Z, fp, spec.ax, spec.by, spec.cz, nx, ny,
                    NSLICE, cfg["radius"])
    return {"V": V, "T": O.transmission(V, 200.0, spec.ax, spec.by, np.complex64),
            "props": [O.propagator_tables(nx, ny, spec.ax, spec.by, 200.0, spec.cz / NSLICE,
                                          precision="f32")] * NSLICE,
            "mask": O.band_mask(nx, ny, spec.ax, spec.by),
            "dm": O.detector_masks(nx, ny, spec.ax, spec.by, cfg["det_k"])}


def cpu_baseline(cfg, nprobe, check=None, prep=None):
    """Oracle port of the reference CPU loop on a bounded probe sample.  With
    `check` (the GPU's detector sums of the same raster) it also reports their
    relative L2 error per detector against this FP32 CPU run."""
    from oracle import msl_oracle as O
    spec = cfg["spec"]
    nx = ny = 512
    workers = os.cpu_count() or 1
    if prep is None:
        prep = cpu_prepare(cfg)
    T, props, mask, dm = prep["T"], prep["props"], prep["mask"], prep["dm"]
    xy = cfg["probe_xy"][:nprobe]
    t0 = time.perf_counter()
    P = O.probe(nx, ny, spec.ax, spec.by, 200.0, 0.0, cfg["k_ap"], 0.0, 0.0, xy, np.complex64)
    det = O.stem(T, props, np.arange(NSLICE), mask, P, dm, [NSLICE - 1], workers=workers)
    el = time.perf_counter() - t0
    res = {"value": nprobe * NSLICE / el, "unit": UNIT, "cores": workers, "kind": "port",
           "sample": f"{nprobe} probes x {NSLICE} slices of the 512^2 SrTiO3 scan "
                     f"(numpy/scipy oracle, FFT workers={workers}), {el:.1f} s"}
    if check is not None:
        # the checker (not timed): the GPU's detector sums for the same probes
        got = np.asarray(check)
        names = ("HAADF", "ABF")
        res["accuracy"] = {
            "rel_l2_vs_cpu_f32": {n: O.rel_l2(got[:nprobe, 0, k], det[:, 0, k]) for k, n in enumerate(names)},
            "probes_f32": nprobe}
    return res


def accuracy_fp64(cfg, xy, got, device_index):
    """The checker (not timed): every probe's HAADF / ABF sum of the timed scan
    against the FP64 oracle (torch complex128 on the same GPU, its own FP64
    potential and transmission functions)."""
    import torch

    from multislice_gb300 import fparams_table
    from oracle import fp64_gpu
    spec = cfg["spec"]
    dev = torch.device("cuda", device_index)
    t0 = time.perf_counter()
    V = fp64_gpu.potential(spec.x, spec.y, spec.z, spec.Z, fparams_table(), spec.ax, spec.by, spec.cz, 512, 512,
                           NSLICE, cfg["radius"], dev)
    T = fp64_gpu.transmission(V, 200.0, spec.ax, spec.by)
    del V
    P = fp64_gpu.propagator(512, 512, spec.ax, spec.by, 200.0, spec.cz / NSLICE, dev)
    ref = fp64_gpu.stem_scan(T, P, np.arange(NSLICE), 512, 512, spec.ax, spec.by, 200.0, cfg["k_ap"], xy,
                             cfg["det_k"], [NSLICE - 1], batch=256)
    del T, P
    torch.cuda.empty_cache()
    from oracle import msl_oracle as O
    names = ("HAADF", "ABF")
    return ({"rel_l2_vs_fp64": {n: O.rel_l2(got[:, 0, k], ref[:, 0, k]) for k, n in enumerate(names)},
             "probes_fp64": int(len(xy)), "fp64_oracle": "torch complex128 on the GPU (oracle/fp64_gpu.py)",
             "fp64_seconds": time.perf_counter() - t0, "bar": 1e-3}, ref)


def _time(fn, steps):
    """Wall time per call of fn() (device work synchronised), after one warm-up call."""
    import torch
    fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / steps


def resident_compare(ctx, cfg, side_probes, steps, which=("streaming", "resident")):
    """The on-chip slice loop against the streaming passes on SrTiO3 at 256^2
    (4 x 4 x 50 cells, the 512^2 scan's 0.061 A pixels), side_probes^2 probes
    x 100 slices."""
    import torch

    from multislice_gb300 import specimen as S
    from oracle import msl_oracle as O
    dev = torch.device("cuda", torch.cuda.current_device())
    names = ("HAADF", "ABF")
    a = 3.905
    spec2 = S.srtio3(4, 4, 50, a)
    v = torch.empty((NSLICE, 256, 256), dtype=torch.float32, device=dev)
    ctx.potential(spec2, 256, 256, NSLICE, cfg["radius"], out=v)
    t2 = torch.empty((NSLICE, 256, 256, 2), dtype=torch.float32, device=dev)
    ctx.transmission(v, spec2.ax, spec2.by, 200.0, out=t2)
    del v
    xy2 = S.raster(1.5 * a, 2.5 * a, 1.5 * a, 2.5 * a, side_probes, side_probes)
    outs = {k: torch.empty((len(xy2), 1, 2), dtype=torch.float64, device=dev) for k in which}
    args2 = (t2, spec2.cz / NSLICE, np.arange(NSLICE), spec2.ax, spec2.by, 200.0, cfg["k_ap"], xy2, cfg["det_k"])
    units = len(xy2) * NSLICE
    res = {"workload": f"SrTiO3 [001] 4x4x50 cells, 256x256 (0.061 A pixels), 100 slices, {len(xy2)} probes",
           "unit": UNIT}
    for k in which:
        el = _time(lambda: ctx.stem_scan(*args2, out=outs[k], resident=(k == "resident")), steps)
        res[k] = units / el
    if len(which) == 2:
        rs, rr = outs["streaming"].cpu().numpy(), outs["resident"].cpu().numpy()
        res["resident_over_streaming"] = res["resident"] / res["streaming"]
        res["hbm_bytes_per_probe_slice"] = {"streaming": 32 * 256 * 256,
                                            "resident": "transmission rows only (8 N^2 per slice per cluster, "
                                                        "shared through L2)"}
        res["rel_l2_resident_vs_streaming"] = {n: O.rel_l2(rr[:, 0, k], rs[:, 0, k]) for k, n in enumerate(names)}
    del t2
    torch.cuda.empty_cache()
    return res


def run_resident(args):
    """--resident: the 256^2 on-chip vs streaming comparison alone (one JSON line)."""
    import torch

    from multislice_gb300 import Context
    torch.cuda.set_device(0)
    side = max(1, int(round(args.probes ** 0.5)))
    with Context(0) as ctx:
        which = ("resident",) if args.resident_only else ("streaming", "resident")
        print(json.dumps(resident_compare(ctx, workload(), side, max(1, args.steps), which)), flush=True)


def run_variants(ctx, cfg, xy, plain, ref64, args, t_dev):
    """The other forms of the scan, timed after the headline (not part of `value`):
    * tensor_core: the same scan with the passes' line DFTs as split-bf16
      contractions on the tensor cores, with its error against the FP64 oracle;
    * closure: 25 slices 4x thicker + the learned closure, as fine-slice-equivalent
      probe-slices/s, with its HAADF / ABF error against the FP64 oracle; it is
      used only when that error is within the bar -- else the fine-slice scan is
      the fallback and `value` stays the plain form's;
    * resident_256: the on-chip slice loop (one 8-CTA cluster per probe) against
      the streaming passes on the same crystal at 256^2 (4 x 4 cells, the same
      0.061 A pixels), 4096 probes x 100 slices;
    * autotune: the pass-family schedule the autotuner measures at 512;
    * ctem_si256: the Si 256^2 CTEM case against the compiled reference;
    * uneven_jobs_256 and frozen_phonon_au2048: the uneven-batch and
      frozen-phonon workloads (jobs_measure, frozen_phonon_measure)."""
    import torch

    from multislice_gb300 import specimen as S
    from multislice_gb300.api import Closure
    from oracle import msl_oracle as O
    spec = cfg["spec"]
    dev = torch.device("cuda", torch.cuda.current_device())
    names = ("HAADF", "ABF")
    out = {}
    # ---- the tensor-core form of the passes (split-bf16 line DFTs on tcgen05)
    o_tc = torch.empty((len(xy), 1, 2), dtype=torch.float64, device=dev)
    ctx.set_schedule(512, 3, 3)
    try:
        el = _time(lambda: ctx.stem_scan(t_dev, spec.cz / NSLICE, np.arange(NSLICE), spec.ax, spec.by, 200.0,
                                         cfg["k_ap"], xy, cfg["det_k"], out=o_tc), max(1, args.steps))
    finally:
        ctx.set_schedule(512, 0, 0)
    d = o_tc.cpu().numpy()
    ent = {"value": len(xy) * NSLICE / el, "unit": UNIT, "schedule": "tensor-core row and column passes",
           "rel_l2_vs_plain": {n: O.rel_l2(d[:, 0, k], plain[:, 0, k]) for k, n in enumerate(names)}}
    if ref64 is not None:
        ent["rel_l2_vs_fp64"] = {n: O.rel_l2(d[:, 0, k], ref64[:, 0, k]) for k, n in enumerate(names)}
        ent["within_bar"] = bool(max(ent["rel_l2_vs_fp64"].values()) <= 1e-3)
    out["tensor_core"] = ent
    del o_tc
    # ---- closure
    wfile = os.path.join(ROOT, "multislice_gb300", "data", "closure_srtio3.npy")
    if os.path.exists(wfile):
        net = Closure(ctx, seed=0)
        net.set_params(np.load(wfile))
        nc = NSLICE // 4
        v = torch.empty((nc, 512, 512), dtype=torch.float32, device=dev)
        ctx.potential(spec, 512, 512, nc, cfg["radius"], out=v)
        tc_ = torch.empty((nc, 512, 512, 2), dtype=torch.float32, device=dev)
        ctx.transmission(v, spec.ax, spec.by, 200.0, out=tc_)
        del v
        res = {}

        def closure_scan():
            res["d"] = ctx.stem_scan_closure(net, tc_, spec.cz / nc, np.arange(nc), spec.ax, spec.by, 200.0,
                                             cfg["k_ap"], xy, cfg["det_k"])

        el = _time(closure_scan, max(1, args.steps))
        coarse = ctx.stem_scan(tc_, spec.cz / nc, np.arange(nc), spec.ax, spec.by, 200.0, cfg["k_ap"], xy,
                               cfg["det_k"])[:, 0, :]
        d = res["d"]
        ent = {"value": len(xy) * NSLICE / el, "unit": UNIT + " (fine-slice equivalent)",
               "coarse_slices": nc, "weights": "multislice_gb300/data/closure_srtio3.npy"}
        if ref64 is not None:
            ent["rel_l2_vs_fp64"] = {n: O.rel_l2(d[:, k], ref64[:, 0, k]) for k, n in enumerate(names)}
            ent["coarse_without_closure_rel_l2_vs_fp64"] = {n: O.rel_l2(coarse[:, k], ref64[:, 0, k])
                                                            for k, n in enumerate(names)}
            ent["within_bar"] = bool(max(ent["rel_l2_vs_fp64"].values()) <= 1e-3)
        ent["rel_l2_vs_plain_fine"] = {n: O.rel_l2(d[:, k], plain[:, 0, k]) for k, n in enumerate(names)}
        ent["used"] = bool(ent.get("within_bar", False))
        ent["fallback"] = "plain fine-slice scan (the headline value)" if not ent["used"] else None
        out["closure"] = ent
        net.close()
        del tc_
        torch.cuda.empty_cache()
    # ---- on-chip slice loop at 256^2
    out["resident_256"] = resident_compare(ctx, cfg, 64, max(1, args.steps))
    # ---- autotuner at 512
    rf, cf, ms = ctx.autotune(512, 128, reps=2)
    fam = ("fast", "tma", "register")
    out["autotune_512"] = {"row": fam[rf], "col": fam[cf],
                           "ms_per_slice_step_128_waves": {f"{fam[i]}/{fam[j]}": float(ms[i, j])
                                                           for i in range(3) for j in range(3)}}
    ctx.set_schedule(512, 0, 0)
    torch.cuda.empty_cache()
    # ---- the CTEM case against the compiled reference
    out["ctem_si256"] = ctem_config1_measure(ctx, max(1, args.steps))
    # ---- the other two workloads: the 256-job uneven batch (every 8th job
    # against FP64 here; --jobs checks all) and the Au 2048^2 frozen-phonon image
    out["uneven_jobs_256"] = jobs_measure(args, fp64_every=8)
    torch.cuda.empty_cache()
    out["frozen_phonon_au2048"] = frozen_phonon_measure()
    return out


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cfg = workload()
    prep = cpu_prepare(cfg)  # the workload's inputs, built once outside the timed steps
    res = None
    times = []
    for i in range(args.warmup + args.steps):
        res = cpu_baseline(cfg, args.cpu_probes, prep=prep)
        if i >= args.warmup:
            times.append(res["value"])
    value = float(np.median(times))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64/f32", "data": "synthetic (SrTiO3 on ideal sites, seeded raster)",
        "impl": "reference",
        "config": {"workload": "SrTiO3 [001] 8x8x50 cells, 512x512, 100 slices, 200 kV, "
                               "25 mrad probe, 64x64 raster (4096 probes), HAADF 80-200 + ABF 11-22 mrad",
                   "sample_probes_per_step": args.cpu_probes},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["cores"], "kind": "port",
                         "sample": res["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_jobs_bench(args):
    """--jobs: the uneven batch with every job checked against FP64; one JSON line."""
    print(json.dumps(jobs_measure(args, fp64_every=1)), flush=True)


def jobs_measure(args, fp64_every=1):
    """The uneven batch of 256 seeded jobs (grid sides 256-1024, 20-300 slices of
    1-2 A, amorphous C/Si/Cu/Au at 0.05 atoms/A^3, 80/200/300 kV, plane waves and
    probes mixed) through msl_run_jobs, once on the FP32 passes and once with the
    tensor-core passes where they are built (sides 256 and 512); the exit waves
    of every `fp64_every`-th job against the FP64 oracle (its own FP64
    potential, transmission and slice loop)."""
    import ctypes

    import torch

    from multislice_gb300 import Context, fparams_table, specimen as S
    from oracle import fp64_gpu
    from oracle import msl_oracle as O
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    descs = S.uneven_jobs(args.jobs_seed, args.njobs)
    gen_s = time.perf_counter() - t0
    fp = fparams_table()
    line = {"workload": f"{args.njobs} uneven jobs (seed {args.jobs_seed}): sides 256-1024, 20-300 slices of 1-2 A, "
                        "amorphous C/Si/Cu/Au 0.05 atoms/A^3, 80/200/300 kV, plane waves and probes",
            "unit": UNIT, "specimen_seconds": gen_s,
            "atoms": int(sum(d["spec"].natom for d in descs)),
            "probe_slices": int(sum(d["nslice"] for d in descs)),
            "sides": {str(n): sum(1 for d in descs if d["n"] == n) for n in (256, 384, 512, 768, 1024)}}
    with Context(0) as ctx:
        jobs = []
        for d in descs:
            s, n = d["spec"], d["n"]
            v = torch.empty((d["nslice"], n, n), dtype=torch.float32, device=dev)
            ctx.potential(s, n, n, d["nslice"], 3.0, out=v)
            t = torch.empty((d["nslice"], n, n, 2), dtype=torch.float32, device=dev)
            ctx.transmission(v, s.ax, s.by, d["kev"], out=t)
            del v
            job = dict(trans=t, ax=s.ax, by=s.by, kev=d["kev"], dz=d["dz"], layer_seq=np.arange(d["nslice"]),
                       out=torch.empty((n, n, 2), dtype=torch.float32, device=dev))
            if d["probe"] is not None:
                job["probe"] = d["probe"]
            jobs.append(job)
        units = line["probe_slices"]
        arms = {}
        for arm in ("fp32", "tensor_core"):
            if arm == "tensor_core":
                ctx.set_schedule(256, 3, 3)
                ctx.set_schedule(512, 3, 3)
            el = _time(lambda: ctx.run_jobs(jobs), max(1, args.steps))
            waves = [j["out"].cpu().numpy() for j in jobs]
            arms[arm] = {"value": units / el, "seconds": el,
                         "algorithmic_gbs": 1e-9 * sum(40 * d["n"] * d["n"] * d["nslice"] for d in descs) / el,
                         "waves": [w[..., 0] + 1j * w[..., 1] for w in waves]}
            ctx.set_schedule(256, 0, 0)
            ctx.set_schedule(512, 0, 0)
        # device time per kind of one FP32 run with per-launch events (the grid
        # groups then run one after another on the context's stream)
        ctx._lib.msl_profile_enable(ctx._h, 1)
        t0 = time.perf_counter()
        ctx.run_jobs(jobs)
        devt = {"serialised_wall_ms": 1e3 * (time.perf_counter() - t0)}
        for k, name in enumerate(("row", "col", "potential", "other")):
            n, ms = ctypes.c_int64(), ctypes.c_double()
            ctx._lib.msl_profile_read(ctx._h, k, ctypes.byref(n), ctypes.byref(ms))
            if n.value:
                devt[name] = {"launches": n.value, "ms": ms.value}
        ctx._lib.msl_profile_enable(ctx._h, 0)
        line["fp32_device_time"] = devt
        # per slice: the wave read and written by both passes (32 N^2) and the
        # job's own transmission layer read once (8 N^2; jobs share no layers)
        line["algorithmic_bytes"] = int(sum(40 * d["n"] * d["n"] * d["nslice"] for d in descs))
        del jobs
        torch.cuda.empty_cache()
        errs = {"fp32": [], "tensor_core": []}
        t1 = time.perf_counter()
        for i, d in enumerate(descs):
            if i % fp64_every:
                continue
            s, n = d["spec"], d["n"]
            V = fp64_gpu.potential(s.x, s.y, s.z, s.Z, fp, s.ax, s.by, s.cz, n, n, d["nslice"], 3.0, dev)
            T = fp64_gpu.transmission(V, d["kev"], s.ax, s.by)
            del V
            P = fp64_gpu.propagator(n, n, s.ax, s.by, d["kev"], d["dz"], dev)
            if d["probe"] is None:
                w0 = torch.ones((n, n), dtype=torch.complex128, device=dev)
            else:
                k_ap, x, y = d["probe"]
                w0 = fp64_gpu.probes(n, n, s.ax, s.by, d["kev"], 0.0, k_ap, 0.0, 0.0, [[x, y]], dev)[0]
            ref = fp64_gpu.multislice(w0, T, P, range(d["nslice"])).cpu().numpy()
            del T
            for arm in errs:
                errs[arm].append(O.rel_l2(arms[arm]["waves"][i], ref))
        torch.cuda.empty_cache()
        line["fp64_seconds"] = time.perf_counter() - t1
    checked = [i for i in range(len(descs)) if i % fp64_every == 0]
    for arm in arms:
        e = np.array(errs[arm])
        arms[arm].pop("waves")
        arms[arm]["rel_l2_vs_fp64"] = {"worst": float(e.max()), "median": float(np.median(e)),
                                       "worst_job": checked[int(e.argmax())], "jobs_checked": len(checked)}
    arms["tensor_core"]["note"] = "tensor-core passes at sides 256 and 512, FP32 passes at 384, 768, 1024"
    line["arms"] = arms
    return line


def run_sides(args):
    """Per-pass device time of the slice loop at every supported side from 256 up
    (batched plane waves, 20 slices over 4 random phase layers, waves larger than
    L2): one JSON line per side with each pass's algorithmic bandwidth and its
    fraction of the measured HBM copy bandwidth."""
    import ctypes

    import torch

    from multislice_gb300 import Context

    hbm, peak_kind = peaks()
    with Context(0) as c:
        for n, batch in ((256, 1024), (384, 512), (512, 256), (768, 128), (1024, 64), (2048, 16)):
            nt = 4
            rng = np.random.default_rng(1)
            t = np.exp(1j * rng.uniform(0, 0.3, (nt, n, n))).astype(np.complex64)
            td = torch.from_numpy(t.view(np.float32).reshape(nt, n, n, 2)).cuda()
            psi = torch.zeros((batch, n, n, 2), dtype=torch.float32, device="cuda")
            psi[..., 0] = 1
            seq = np.arange(20) % nt
            dz = np.full(nt, 1.5)
            for _ in range(max(args.warmup, 3)):
                c.multislice(td, dz, seq, 20.0, 20.0, 200.0, psi=psi)
            torch.cuda.synchronize()
            c._lib.msl_profile_enable(c._h, 1)
            for _ in range(max(args.steps, 1)):
                c.multislice(td, dz, seq, 20.0, 20.0, 200.0, psi=psi)
            torch.cuda.synchronize()
            line = {"side": n, "batch": batch, "peak_gbs": hbm, "peak_source": peak_kind}
            for k, name in ((0, "row"), (1, "col")):
                cnt, ms = ctypes.c_int64(), ctypes.c_double()
                c._lib.msl_profile_read(c._h, k, ctypes.byref(cnt), ctypes.byref(ms))
                per = ms.value / max(cnt.value, 1)
                gbs = 16.0 * n * n * batch / (per * 1e-3) / 1e9
                line[name] = {"ms_per_launch": per, "achieved_gbs": gbs, "frac": gbs / hbm}
            c._lib.msl_profile_enable(c._h, 0)
            print(json.dumps(line), flush=True)
            del psi, td
            torch.cuda.empty_cache()


def run_potential(args):
    """--potential: the projected potential of one Au 2048^2 configuration (fcc Au
    16x16x40 cells, 80 slices, 3 A cutoff; the frozen-phonon workload's
    per-configuration build) through msl_potential_build into device memory:
    device time per launch (CUDA events on the library stream) and the pair
    evaluations it makes (pixel-atom pairs inside the cutoff)."""
    import ctypes

    import torch

    from multislice_gb300 import Context, specimen as S

    spec = S.jitter(S.fcc_au(), 0.085, np.random.default_rng(7))
    n, nslice, radius = 2048, 80, 3.0
    v = torch.empty((nslice, n, n), dtype=torch.float32, device="cuda:0")
    with Context(0) as c:
        c.potential(spec, n, n, nslice, radius, out=v)
        c._lib.msl_profile_enable(c._h, 1)
        reps = max(1, args.steps)
        for _ in range(reps):
            c.potential(spec, n, n, nslice, radius, out=v)
        k, ms = ctypes.c_int64(), ctypes.c_double()
        c._lib.msl_profile_read(c._h, 2, ctypes.byref(k), ctypes.byref(ms))
        c._lib.msl_profile_enable(c._h, 0)
    dxp = spec.ax / n
    pairs_per_pixel = np.pi * radius ** 2 * spec.natom / nslice / (spec.ax * spec.by)
    pairs = pairs_per_pixel * n * n * nslice
    line = {"workload": "Au fcc 16x16x40 (40,960 atoms, jittered 0.085 A), 2048^2, 80 slices, 3 A cutoff",
            "ms_per_launch": ms.value / max(k.value, 1), "launches": k.value,
            "pixel_size_A": dxp, "pairs_inside_cutoff": pairs,
            "pairs_per_s": pairs / (ms.value / max(k.value, 1) * 1e-3)}
    print(json.dumps(line), flush=True)


def run_ctem(args):
    """--ctem: the Si 256^2 CTEM case; one JSON line."""
    import torch

    from multislice_gb300 import Context
    torch.cuda.set_device(0)
    with Context(0) as ctx:
        print(json.dumps(ctem_config1_measure(ctx, max(1, args.steps))), flush=True)


def ctem_config1_measure(ctx, steps):
    """The CTEM case (Si [001] 5x5x20 cells, 256^2, 80 slices of a/4, 200 kV
    plane wave): the chain potential -> transmission -> slice loop from host
    atoms to the host exit wave, the slice loop alone on device buffers, and the
    exit wave against Kirkland's mulslice compiled from the reference sources
    (the committed golden wave)."""
    import torch

    from multislice_gb300 import specimen as S
    from oracle import msl_oracle as O
    cfg = S.config_si_ctem()
    spec, n, ns, kev = cfg["spec"], cfg["nx"], cfg["nslice"], cfg["kev"]
    gold = np.load(os.path.join(ROOT, "tests", "golden", "si_config1.npz"))["wave"]
    res = {}

    def chain():
        v = ctx.potential(spec, n, n, ns, cfg["radius"])
        t = ctx.transmission(v, spec.ax, spec.by, kev)
        res["w"] = ctx.multislice(t, spec.cz / ns, np.arange(ns), spec.ax, spec.by, kev)[0]

    e2e = _time(chain, steps)
    dev = torch.device("cuda", torch.cuda.current_device())
    v = torch.empty((ns, n, n), dtype=torch.float32, device=dev)
    ctx.potential(spec, n, n, ns, cfg["radius"], out=v)
    t = torch.empty((ns, n, n, 2), dtype=torch.float32, device=dev)
    ctx.transmission(v, spec.ax, spec.by, kev, out=t)
    psi = torch.empty((1, n, n, 2), dtype=torch.float32, device=dev)

    def loop():
        psi[..., 0] = 1.0
        psi[..., 1] = 0.0
        ctx.multislice(t, spec.cz / ns, np.arange(ns), spec.ax, spec.by, kev, psi=psi)

    dt = _time(loop, steps)
    return {"workload": "Si [001] 5x5x20 cells, 256^2, 80 slices (a/4), 200 kV plane wave",
            "e2e_ms": 1e3 * e2e, "chain": "host atoms -> potential -> transmission -> slice loop -> host wave",
            "slice_loop_ms": 1e3 * dt, "slices_per_s": ns / dt,
            "rel_l2_vs_compiled_reference": O.rel_l2(res["w"], gold),
            "reference": "Kirkland's mulslice compiled from the reference sources (tests/golden/si_config1.npz)"}


def run_frozen_phonon(args):
    """--frozen-phonon: the Au 2048^2 frozen-phonon image; one JSON line."""
    print(json.dumps(frozen_phonon_measure()), flush=True)


def frozen_phonon_measure():
    """The Au 2048^2 frozen-phonon image (fcc Au 16x16x40 cells, 80 slices, 32
    configurations, 300 kV, Cs 1.2 mm, defocus -60 nm, 25 mrad objective
    aperture): wall time of one msl_frozen_phonon call after a warm-up call, and
    the device time per kind (row / column passes, potentials, other)."""
    import ctypes

    from multislice_gb300 import Context, specimen as S

    spec = S.fcc_au()
    kev = 300.0
    k_obj = float(S.mrad_to_k(25.0, kev))
    with Context(0) as c:
        c.frozen_phonon(spec, 2048, 2048, 80, 3.0, kev, 1.2e7, -600.0, k_obj, nconfig=2, sigma=0.085, seed=1)
        t0 = time.perf_counter()
        c.frozen_phonon(spec, 2048, 2048, 80, 3.0, kev, 1.2e7, -600.0, k_obj, nconfig=32, sigma=0.085, seed=2026)
        wall = time.perf_counter() - t0
        line = {"workload": "Au fcc 16x16x40, 2048^2, 80 slices, 32 frozen-phonon configurations, 300 kV",
                "wall_ms": 1e3 * wall, "device_ms_by_kind": "a second call with per-launch events"}
        c._lib.msl_profile_enable(c._h, 1)
        t0 = time.perf_counter()
        c.frozen_phonon(spec, 2048, 2048, 80, 3.0, kev, 1.2e7, -600.0, k_obj, nconfig=32, sigma=0.085, seed=2026)
        line["profiled_wall_ms"] = 1e3 * (time.perf_counter() - t0)
        for k, name in enumerate(("row", "col", "potential", "other")):
            n, ms = ctypes.c_int64(), ctypes.c_double()
            c._lib.msl_profile_read(c._h, k, ctypes.byref(n), ctypes.byref(ms))
            line[name] = {"launches": n.value, "ms": ms.value}
        c._lib.msl_profile_enable(c._h, 0)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-probes", type=int, default=32)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--probes", type=int, default=4096,
                    help="probes of the 64x64 raster per GPU (smaller cases are for profiling)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 accuracy check of every probe")
    ap.add_argument("--jobs", action="store_true",
                    help="the 256-job uneven batch, FP32 and tensor-core arms, each against FP64")
    ap.add_argument("--njobs", type=int, default=256)
    ap.add_argument("--jobs-seed", type=int, default=2026)
    ap.add_argument("--tc", action="store_true",
                    help="run the timed scan on the tensor-core passes (profiling; the headline uses the FP32 passes)")
    ap.add_argument("--resident", action="store_true",
                    help="time the on-chip slice loop against the streaming passes at 256^2 (--probes probes)")
    ap.add_argument("--resident-only", action="store_true", help="with --resident: the on-chip loop alone")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the closure, on-chip and autotuner forms reported beside the headline")
    ap.add_argument("--batch", type=int, default=0, help="probes per launch (0: library default)")
    ap.add_argument("--sides", action="store_true",
                    help="per-pass bandwidth of the slice loop at every side instead of the scan")
    ap.add_argument("--ctem", action="store_true",
                    help="time the Si 256^2 CTEM case and check it against the compiled reference's wave")
    ap.add_argument("--potential", action="store_true",
                    help="time the potential of one Au 2048^2 frozen-phonon configuration")
    ap.add_argument("--frozen-phonon", action="store_true",
                    help="time the Au 2048^2, 32-configuration frozen-phonon image instead of the scan")
    args = ap.parse_args()
    if args.jobs:
        run_jobs_bench(args)
    elif args.resident:
        run_resident(args)
    elif args.sides:
        run_sides(args)
    elif args.frozen_phonon:
        run_frozen_phonon(args)
    elif args.potential:
        run_potential(args)
    elif args.ctem:
        run_ctem(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
