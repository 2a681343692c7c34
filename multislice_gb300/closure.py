"""Training data and training loop of the learned coarse-slice closure.

The closure (msl_closure_* in libmsl.so) corrects an exit wave computed with
slices four times thicker than the fine slicing toward the fine-slice exit
wave.  Its training pairs are produced by the library itself on the specimen
generators of the two benchmark workloads:

  * SrTiO3 [001] (the 512^2 STEM scan's crystal): 4 x 4 cells at 256^2 -- the
    scan's pixel size, 0.061 A -- 50 cells thick, fine slices of a / 2 =
    1.9525 A (the scan's slicing), coarse slices of 7.81 A;
  * diamond-cubic Si [001] (the CTEM workload's crystal): 3 x 3 cells at 256^2
    (0.064 A pixels), 20 cells thick, fine slices of a / 4 = 1.358 A, coarse
    slices of 5.43 A;

each with frozen-phonon displacements for variety and converged 25 mrad
probes at random positions, 200 kV.  Every pair is (coarse exit wave, fine
exit wave) of the same probe through the same atoms.  Training runs the
library's own forward and backward kernels and its Adam step; torch only holds
the pairs in device memory.
"""
from __future__ import annotations

import numpy as np

from . import specimen as S
from .api import Closure, phonon_displacements

KEV = 200.0


def _family(name):
    if name == "srtio3":
        a = 3.905
        return dict(spec=S.srtio3(4, 4, 50, a), n=256, nfine=100, cell=a)
    if name == "si":
        a = 5.431
        return dict(spec=S.si_diamond(3, 3, 20, a), n=256, nfine=80, cell=a)
    raise ValueError(name)


def make_pairs(ctx, n_pairs, seed=0, family="srtio3", nconfig=8, sigma=0.07, radius=3.0, device=None):
    """(coarse, fine) exit waves as torch float32 device tensors [n_pairs, n, n, 2]."""
    import torch

    F = _family(family)
    spec, n, nfine = F["spec"], F["n"], F["nfine"]
    ncoarse = nfine // 4
    dev = device or torch.device("cuda", torch.cuda.current_device())
    coarse = torch.empty((n_pairs, n, n, 2), dtype=torch.float32, device=dev)
    fine = torch.empty_like(coarse)
    rng = np.random.default_rng(seed)
    k_ap = float(S.mrad_to_k(25.0, KEV))
    per = [n_pairs // nconfig + (1 if i < n_pairs % nconfig else 0) for i in range(nconfig)]
    p0 = 0
    for c in range(nconfig):
        if per[c] == 0:
            continue
        d = phonon_displacements(seed * 1000 + c, c, spec.natom, sigma)
        js = S.Specimen(spec.x + d[:, 0], spec.y + d[:, 1], spec.z + d[:, 2], spec.Z, spec.ax, spec.by, spec.cz)
        xy = np.stack([rng.uniform(0, spec.ax, per[c]), rng.uniform(0, spec.by, per[c])], axis=1)
        for ns, dst in ((nfine, fine), (ncoarse, coarse)):
            v = torch.empty((ns, n, n), dtype=torch.float32, device=dev)
            ctx.potential(js, n, n, ns, radius, out=v)
            t = torch.empty((ns, n, n, 2), dtype=torch.float32, device=dev)
            ctx.transmission(v, spec.ax, spec.by, KEV, out=t)
            ctx.stem_exit_waves(t, spec.cz / ns, np.arange(ns), spec.ax, spec.by, KEV, k_ap, xy,
                                out=dst[p0:p0 + per[c]])
            del v, t
        p0 += per[c]
    return coarse, fine


def rel_error(a, b):
    """sqrt(sum |a - b|^2 / sum |b|^2) over whole stacks (torch tensors)."""
    import torch
    return float(torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double()))


def evaluate(net, coarse, fine, batch=16):
    """(error of the coarse waves, error after the closure) against the fine ones."""
    import torch
    corr = coarse.clone()
    for i in range(0, len(corr), batch):
        net.apply(corr[i:i + batch])
    torch.cuda.synchronize()
    return rel_error(coarse, fine), rel_error(corr, fine)


def train(ctx, net, coarse, fine, steps, batch=8, lr=1e-3, seed=0, lr_final=None, log=None, log_every=100):
    """Adam steps on random minibatches of the pairs; returns the loss history."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for it in range(steps):
        lr_t = lr if lr_final is None else lr * (lr_final / lr) ** (it / max(steps - 1, 1))
        idx = torch.randint(0, len(coarse), (batch,), generator=g).to(coarse.device)
        cb = coarse.index_select(0, idx).contiguous()
        fb = fine.index_select(0, idx).contiguous()
        loss = net.train_step(cb, fb, lr_t)
        hist.append(loss)
        if log is not None and (it % log_every == 0 or it == steps - 1):
            log(f"step {it} loss {loss:.4e} lr {lr_t:.2e}")
    return hist


__all__ = ["Closure", "make_pairs", "train", "evaluate", "rel_error"]
