"""Train the learned coarse-slice closure on pairs the library makes, and judge it
on the 512^2 SrTiO3 STEM scan against the fine-slice scan.

    python -m multislice_gb300.train_closure --pairs 20000 --steps 4000 \
        --out closure_srtio3.npy --log closure_train.json

Steps: (1) training pairs (multislice_gb300.closure.make_pairs: SrTiO3 and Si,
frozen-phonon configurations, random probe positions, fine slices vs 4x
thicker ones, 256^2); (2) Adam on random minibatches with the library's own
forward / backward kernels, validation on held-out pairs; (3) the judge: the
SrTiO3 8x8x50-cell 512^2 scan over `--judge-probes` probes of the 64x64 raster
with the fine slicing (100 slices), the coarse slicing (25 slices) without and
with the closure -- HAADF / ABF relative L2 errors of the coarse and closure
images against the fine one.  The weights (FP32, the library's parameter
layout) and a JSON log are written out.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def judge(ctx, net, nprobe=256, seed=0):
    """Fine vs coarse vs coarse + closure on the benchmark scan's first probes."""
    import torch

    from . import specimen as S
    cfg = S.config_srtio3_stem()
    spec = cfg["spec"]
    xy = cfg["probe_xy"][:: max(1, len(cfg["probe_xy"]) // nprobe)][:nprobe]
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {}
    for ns in (100, 25):
        v = torch.empty((ns, 512, 512), dtype=torch.float32, device=dev)
        ctx.potential(spec, 512, 512, ns, cfg["radius"], out=v)
        t = torch.empty((ns, 512, 512, 2), dtype=torch.float32, device=dev)
        ctx.transmission(v, spec.ax, spec.by, 200.0, out=t)
        del v
        d = ctx.stem_scan(t, spec.cz / ns, np.arange(ns), spec.ax, spec.by, 200.0, cfg["k_ap"], xy, cfg["det_k"])
        out[ns] = d[:, 0, :]
        if ns == 25:
            out["closure"] = ctx.stem_scan_closure(net, t, spec.cz / ns, np.arange(ns), spec.ax, spec.by, 200.0,
                                                   cfg["k_ap"], xy, cfg["det_k"])
        del t
        torch.cuda.empty_cache()

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    res = {}
    for k, name in enumerate(("HAADF", "ABF")):
        res[name] = {"coarse_vs_fine": rel(out[25][:, k], out[100][:, k]),
                     "closure_vs_fine": rel(out["closure"][:, k], out[100][:, k])}
    res["probes"] = int(len(xy))
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--si-fraction", type=float, default=0.25)
    ap.add_argument("--val", type=int, default=256)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--judge-probes", type=int, default=256)
    ap.add_argument("--init", default=None, help="start from these weights (.npy)")
    ap.add_argument("--out", default="closure_srtio3.npy")
    ap.add_argument("--log", default="closure_train.json")
    args = ap.parse_args(argv)

    import torch

    from . import closure as CL
    from .api import Closure, Context

    torch.cuda.set_device(0)
    log = {"args": vars(args)}
    with Context(0) as ctx:
        t0 = time.perf_counter()
        n_si = int(args.pairs * args.si_fraction)
        parts = [CL.make_pairs(ctx, args.pairs - n_si, seed=args.seed, family="srtio3")]
        if n_si:
            parts.append(CL.make_pairs(ctx, n_si, seed=args.seed + 1, family="si"))
        coarse = torch.cat([p[0] for p in parts])
        fine = torch.cat([p[1] for p in parts])
        del parts
        perm = torch.randperm(len(coarse), generator=torch.Generator().manual_seed(args.seed)).to(coarse.device)
        coarse, fine = coarse[perm].contiguous(), fine[perm].contiguous()
        va_c, va_f = coarse[:args.val].contiguous(), fine[:args.val].contiguous()
        tr_c, tr_f = coarse[args.val:].contiguous(), fine[args.val:].contiguous()
        del coarse, fine
        torch.cuda.synchronize()
        log["pairs_seconds"] = time.perf_counter() - t0
        net = Closure(ctx, seed=args.seed)
        if args.init:
            net.set_params(np.load(args.init))
        e0, e_before = CL.evaluate(net, va_c, va_f)
        t1 = time.perf_counter()
        hist = CL.train(ctx, net, tr_c, tr_f, args.steps, batch=args.batch, lr=args.lr, lr_final=args.lr_final,
                        seed=args.seed, log=print, log_every=500)
        torch.cuda.synchronize()
        log["train_seconds"] = time.perf_counter() - t1
        log["steps_per_second"] = args.steps / log["train_seconds"]
        _, e_after = CL.evaluate(net, va_c, va_f)
        log["validation"] = {"coarse_vs_fine": e0, "initial_net_vs_fine": e_before, "closure_vs_fine": e_after}
        log["loss_first_last"] = [hist[0], float(np.mean(hist[-50:]))]
        del tr_c, tr_f, va_c, va_f
        torch.cuda.empty_cache()
        np.save(args.out, net.get_params())
        log["judge_512_scan"] = judge(ctx, net, args.judge_probes)
        net.close()
    with open(args.log, "w") as f:
        json.dump(log, f, indent=1)
    print(json.dumps(log))


if __name__ == "__main__":
    main()
