"""FP64 multislice oracle on the GPU (torch complex128) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg (its
accuracy check) may import this module, and only as the checker, never as the
product path (the product is libmsl.so, include/msl.h).

The same restatement of the reference's algorithm as oracle/msl_oracle.py in
its complex128 form -- Kirkland's vzatom potential with FPARAMS coefficients
(slicelib.cpp:2666-2716, Bessel functions :168-235) binned and cut off as
LMultiSlice does (ModelPotential.cu:27-99, :154-203), t = exp(i sigma V)
band-limited by fft -> mask -> ifft (mulslice.cpp:414-421, :515-522), the slice
loop wave *= t; fft; propagate; ifft (mulslice.cpp:706-739) with the separable
propagator (slicelib.cpp:744-790), the C# probe and annular detector
(MSProject.cs:458-514, :792-842) and the objective lens (mulslice.cpp:539-676)
-- with every step in FP64, batched over probes or configurations, so that
full-size workloads (thousands of 512^2 probes, 2048^2 frozen-phonon images)
get an FP64 reference on every pixel in seconds.  It runs on any torch device;
tests/test_oracle_fp64.py pins it against msl_oracle on the CPU.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import msl_oracle as O

F64 = torch.float64
C128 = torch.complex128


def _horner(coefs, t):
    s = torch.full_like(t, coefs[-1])
    for c in coefs[-2::-1]:
        s = s * t + c
    return s


def bessk0(x):
    """K0 of A&S 9.8.5-9.8.6 (slicelib.cpp:210-235) for x > 0."""
    small = x <= 2.0
    xs = torch.where(small, x, torch.ones_like(x))
    t = (xs / 3.75) ** 2
    i0 = _horner(O._I0A, t)  # xs <= 2 < 3.75: the small-argument I0 branch
    s_s = -torch.log(xs / 2.0) * i0 + _horner(O._K0A, (xs / 2.0) ** 2)
    xl = torch.where(small, torch.full_like(x, 3.0), x)
    s_l = torch.exp(-xl) * _horner(O._K0B, 2.0 / xl) / torch.sqrt(xl)
    return torch.where(small, s_s, s_l)


def vzatom(p, r):
    """vzatom (slicelib.cpp:2666-2716); p [n, 12] coefficient rows, r [n, ...] > 0."""
    shp = (-1,) + (1,) * (r.dim() - 1)
    q = [p[:, i].reshape(shp) for i in range(12)]
    x = 2.0 * O.PI_K * r
    suml = (q[0] * bessk0(x * torch.sqrt(q[1])) + q[2] * bessk0(x * torch.sqrt(q[3]))
            + q[4] * bessk0(x * torch.sqrt(q[5])))
    x2 = (O.PI_K * r) ** 2
    sumg = (q[6] * torch.exp(-x2 / q[7]) / q[7] + q[8] * torch.exp(-x2 / q[9]) / q[9]
            + q[10] * torch.exp(-x2 / q[11]) / q[11])
    return O.AL * suml + O.AG * sumg


def potential(x, y, z, Znum, fparams, ax, by, cz_total, nx, ny, nslice, radius, device, chunk=1024):
    """V_z per slice, float64 [nslice, nx, ny] on `device` (msl_oracle.potential)."""
    if 2.0 * radius >= ax or 2.0 * radius >= by:
        raise ValueError("cutoff radius must be below half the cell")
    kz = O.slice_index(z, cz_total, nslice)
    keep = kz >= 0
    x, y, Znum, kz = (np.asarray(v)[keep] for v in (x, y, Znum, kz))
    dxp, dyp = ax / nx, by / ny
    wx = min(nx, int(math.ceil(2 * radius / dxp)) + 3)
    wy = min(ny, int(math.ceil(2 * radius / dyp)) + 3)
    out = torch.zeros(nslice * nx * ny, dtype=F64, device=device)
    fp = torch.as_tensor(np.asarray(fparams, np.float64), device=device)
    ox = torch.arange(wx, device=device, dtype=torch.int64)
    oy = torch.arange(wy, device=device, dtype=torch.int64)
    for a0 in range(0, len(x), chunk):
        xa = torch.as_tensor(np.asarray(x[a0:a0 + chunk], np.float64), device=device)
        ya = torch.as_tensor(np.asarray(y[a0:a0 + chunk], np.float64), device=device)
        xa = xa - ax * torch.floor(xa / ax)
        ya = ya - by * torch.floor(ya / by)
        Z = torch.as_tensor(np.asarray(Znum[a0:a0 + chunk], np.int64), device=device)
        k = torch.as_tensor(np.asarray(kz[a0:a0 + chunk], np.int64), device=device)
        if wx < nx:
            ix = (torch.floor((xa - radius) / dxp).long() - 1)[:, None] + ox[None, :]
        else:
            ix = ox[None, :].expand(len(xa), -1)
        if wy < ny:
            iy = (torch.floor((ya - radius) / dyp).long() - 1)[:, None] + oy[None, :]
        else:
            iy = oy[None, :].expand(len(ya), -1)
        ix = torch.remainder(ix, nx)
        iy = torch.remainder(iy, ny)
        ddx = torch.abs(xa[:, None] - ix.to(F64) * dxp)
        ddx = torch.where(ddx >= ax / 2.0, ax - ddx, ddx)
        ddy = torch.abs(ya[:, None] - iy.to(F64) * dyp)
        ddy = torch.where(ddy >= by / 2.0, by - ddy, ddy)
        r = torch.sqrt(ddx[:, :, None] ** 2 + ddy[:, None, :] ** 2)
        inside = r < radius
        v = vzatom(fp[Z], torch.clamp(r, min=1.0e-10))
        v = torch.where(inside, v, torch.zeros_like(v))
        idx = (k[:, None, None] * nx + ix[:, :, None]) * ny + iy[:, None, :]
        out.index_add_(0, idx.reshape(-1), v.reshape(-1))
    return out.reshape(nslice, nx, ny)


def kfft(w):
    """Kirkland fft: exp(+i..) unscaled over the last two axes."""
    return torch.fft.ifft2(w, norm="forward")


def kifft(w):
    """Kirkland ifft: exp(-i..) scaled by 1/(nx ny)."""
    return torch.fft.fft2(w, norm="forward")


def band_mask(nx, ny, ax, by, device, bw=2.0 / 3.0):
    return torch.as_tensor(O.band_mask(nx, ny, ax, by, bw), device=device)


def transmission(V, kev, ax, by, bw=2.0 / 3.0):
    """Band-limited exp(i sigma V) per layer, complex128 (FP64 phase)."""
    nl, nx, ny = V.shape
    t = torch.exp(1j * (O.sigma(kev) / 1000.0) * V.to(F64))
    m = band_mask(nx, ny, ax, by, V.device, bw)
    return kifft(torch.where(m, kfft(t), torch.zeros((), dtype=C128, device=V.device)))


def propagator(nx, ny, ax, by, kev, dz, device, bw=2.0 / 3.0, tilt=(0.0, 0.0)):
    """px py and the band limit folded into one [nx, ny] complex128 table."""
    px, py = O.propagator_tables(nx, ny, ax, by, kev, dz, ctilt=tilt, precision="f64")
    P = np.where(O.band_mask(nx, ny, ax, by, bw), px[:, None] * py[None, :], 0)
    return torch.as_tensor(P, dtype=C128, device=device)


def probes(nx, ny, ax, by, kev, k_in, k_out, df, cs, xy, device):
    """Converged probes in real space, complex128 [nprobe, nx, ny] (MSProject.cs:458-514)."""
    lam = O.wavelength(kev)
    kxd, kyd = (torch.as_tensor(v, dtype=F64, device=device) for v in O.k_tables_f64(nx, ny, ax, by))
    s = kxd[:, None] ** 2 + kyd[None, :] ** 2
    ap = (s >= k_in ** 2) & (s <= k_out ** 2)
    chi = math.pi * (lam * df * s + 0.5 * cs * lam ** 3 * s * s)
    i = torch.as_tensor(O.signed_index(nx), dtype=F64, device=device)[:, None]
    j = torch.as_tensor(O.signed_index(ny), dtype=F64, device=device)[None, :]
    xy = torch.as_tensor(np.atleast_2d(np.asarray(xy, np.float64)), device=device)
    ph = 2.0 * math.pi * (i[None] * (xy[:, 0, None, None] / ax) + j[None] * (xy[:, 1, None, None] / by)) - chi[None]
    P = torch.where(ap[None], torch.exp(1j * ph), torch.zeros((), dtype=C128, device=device))
    return kifft(P)


def detector_masks(nx, ny, ax, by, det_k, device):
    return torch.as_tensor(O.detector_masks(nx, ny, ax, by, det_k), dtype=F64, device=device)


def stem(T, prop, layer_seq, P0, dmask, checkpoints):
    """Detector sums [nprobe, ncheck, ndet] of probes P0 through layers T (FP64).

    prop: one [nx, ny] table, or a list of them per layer."""
    props = prop if isinstance(prop, (list, tuple)) else [prop] * T.shape[0]
    w = P0.clone()
    out = []
    last = checkpoints[-1]
    for s, l in enumerate(layer_seq):
        W = kfft(w * T[l]) * props[l]
        if s in checkpoints:
            out.append(torch.einsum("bxy,dxy->bd", W.real ** 2 + W.imag ** 2, dmask))
            if s == last:
                break
        w = kifft(W)
    return torch.stack(out, dim=1)


def stem_scan(T, prop, layer_seq, nx, ny, ax, by, kev, k_ap, xy, det_k, checkpoints, batch=64, k_ap_in=0.0,
              df=0.0, cs=0.0):
    """The whole scan in probe batches; returns numpy float64 [nprobe, ncheck, ndet]."""
    dev = T.device
    dm = detector_masks(nx, ny, ax, by, det_k, dev)
    xy = np.atleast_2d(np.asarray(xy, np.float64))
    res = []
    for p0 in range(0, len(xy), batch):
        P0 = probes(nx, ny, ax, by, kev, k_ap_in, k_ap, df, cs, xy[p0:p0 + batch], dev)
        res.append(stem(T, prop, layer_seq, P0, dm, list(checkpoints)).cpu().numpy())
    return np.concatenate(res, axis=0)


def multislice(w, T, prop, layer_seq):
    """Exit waves of wave(s) w through layers T (FP64)."""
    props = prop if isinstance(prop, (list, tuple)) else [prop] * T.shape[0]
    for l in layer_seq:
        w = kifft(kfft(w * T[l]) * props[l])
    return w


def ctf(nx, ny, ax, by, kev, cs, df, k_obj, device, astig=(0.0, 0.0, 0.0, 0.0)):
    return torch.as_tensor(O.ctf(nx, ny, ax, by, kev, cs, df, k_obj, astig=astig), device=device)


def frozen_phonon(spec, fparams, nx, ny, nslice, radius, kev, cs, df, k_obj, nconfig, sigma, seed, device,
                  cfg_batch=4):
    """Configuration-averaged CTEM image and exit intensity (FP64), numpy [nx, ny]
    each: displacements of the library's stream (msl_oracle.phonon_displacements)."""
    P = propagator(nx, ny, spec.ax, spec.by, kev, spec.cz / nslice, device)
    C = ctf(nx, ny, spec.ax, spec.by, kev, cs, df, k_obj, device)
    img = torch.zeros((nx, ny), dtype=F64, device=device)
    exi = torch.zeros((nx, ny), dtype=F64, device=device)
    for c in range(nconfig):
        d = O.phonon_displacements(seed, c, spec.natom, sigma)
        V = potential(spec.x + d[:, 0], spec.y + d[:, 1], spec.z + d[:, 2], spec.Z, fparams, spec.ax, spec.by,
                      spec.cz, nx, ny, nslice, radius, device)
        T = transmission(V, kev, spec.ax, spec.by)
        del V
        w = multislice(torch.ones((nx, ny), dtype=C128, device=device), T, P, range(nslice))
        del T
        exi += (w.real ** 2 + w.imag ** 2) / nconfig
        im = kifft(kfft(w) * C)
        img += (im.real ** 2 + im.imag ** 2) / nconfig
    return img.cpu().numpy(), exi.cpu().numpy()
