"""CPU oracle for the multislice hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module, and only as the checker (or the timed CPU baseline), never as the
product path.  The product is libmsl.so (include/msl.h).

A numpy restatement of the reference's algorithm, in Kirkland's conventions:

* FFT: Kirkland's "fft" is FFTW_BACKWARD (exp(+i..)) unscaled and his "ifft" is
  FFTW_FORWARD (exp(-i..)) scaled by 1/(nx*ny)   (multislice/cfpix.cpp:115-230).
* Layout: x-major, element (ix, iy) at iy + ix*ny   (cfpix.hpp:99-125).
* Potential: Kirkland's vzatom() functional form (multislice/slicelib.cpp:2666-2716,
  Bessel K0/I0 of Abramowitz & Stegun 9.8.1-9.8.6 at :168-235) with the
  reference's FPARAMS.DAT coefficients, summed in real space per slice with the
  z-binning, single minimum image and strict cutoff of LMultiSlice
  (ImageSimulation/LMultiSlice/ModelPotential.cu:27-99, :125-230).
* Transmission: t = exp(i*sigma*V_z) band-limited to k < (2/3) k_Nyquist by
  fft -> mask -> ifft   (multislice/mulslice.cpp:414-421, :481-489, :515-522).
* Propagator: separable px(kx)*py(ky) with py applied first, zero outside the
  same band limit   (mulslice.cpp:494-513, slicelib.cpp:744-790).
* Slice loop: wave *= t; fft; propagate; ifft   (mulslice.cpp:706-739).
* STEM: probe of MSProject.cs:458-514, detection after the propagator of each
  checkpoint slice (MSReuseCalculator.cs:36-92), annular sums with inclusive
  bounds (MSProject.cs:792-842).  The C# code works in the complex-conjugate
  convention of Kirkland's; every intensity is identical, so the probe here is
  the conjugate of the C# probe and the loop is Kirkland's.

Two precisions: ``complex64`` mirrors Kirkland's single-precision arithmetic
(float tables built as mulslice.cpp builds them); ``complex128`` is the FP64
oracle (all phase arguments and tables in double).

Pinning: tests/test_oracle_golden.py checks this module against golden vectors
produced by the reference's own compiled code (oracle/ref, see
tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np

try:  # scipy.fft gives multi-threaded transforms for the CPU baseline
    import scipy.fft as _sfft
except Exception:  # pragma: no cover
    _sfft = None

EMASS_KEV = 510.99906      # slicelib.cpp:2800
HC_KEV_A = 12.3984244      # slicelib.cpp:2801
AL = 300.8242834           # slicelib.cpp:2673 (Lorentzian prefactor)
AG = 150.4121417           # slicelib.cpp:2673 (Gaussian prefactor)
PI_K = 3.141592654         # slicelib.cpp:2674

_I0A = (1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.0360768, 0.0045813)
_I0B = (0.39894228, 0.01328592, 0.00225319, -0.00157565, 0.00916281, -0.02057706,
        0.02635537, -0.01647633, 0.00392377)
_K0A = (-0.57721566, 0.42278420, 0.23069756, 0.03488590, 0.00262698, 0.00010750, 0.00000740)
_K0B = (1.25331414, -0.07832358, 0.02189568, -0.01062446, 0.00587872, -0.00251540, 0.00053208)


# ----------------------------------------------------------------- constants
def wavelength(kev):
    """Electron wavelength in Angstrom (slicelib.cpp:2795-2806)."""
    return HC_KEV_A / np.sqrt(kev * (2.0 * EMASS_KEV + kev))


def sigma(kev):
    """Interaction constant in rad/(kV*Angstrom) (slicelib.cpp:2387-2412)."""
    x = (EMASS_KEV + kev) / (2.0 * EMASS_KEV + kev)
    return 2.0 * (4.0 * np.arctan(1.0)) * x / (wavelength(kev) * kev)


# ----------------------------------------------------------------- potential
def _horner(coefs, t):
    s = np.full_like(t, coefs[-1])
    for c in coefs[-2::-1]:
        s = s * t + c
    return s


def bessi0(x):
    """Modified Bessel I0, A&S 9.8.1-9.8.2 (slicelib.cpp:168-196)."""
    x = np.asarray(x, dtype=np.float64)
    ax = np.abs(x)
    small = ax <= 3.75
    t_s = (x / 3.75) ** 2
    t_l = 3.75 / np.where(small, 1.0, ax)
    s_s = _horner(_I0A, t_s)
    s_l = _horner(_I0B, t_l) * np.exp(np.where(small, 0.0, ax)) / np.sqrt(np.where(small, 1.0, ax))
    return np.where(small, s_s, s_l)


def bessk0(x):
    """Modified Bessel K0, A&S 9.8.5-9.8.6 (slicelib.cpp:210-235)."""
    x = np.asarray(x, dtype=np.float64)
    ax = np.abs(x)
    small = ax <= 2.0
    axs = np.where(small & (ax > 0), ax, 1.0)
    x2 = (axs / 2.0) ** 2
    s_s = -np.log(axs / 2.0) * bessi0(axs) + _horner(_K0A, x2)
    axl = np.where(small, 3.0, ax)
    s_l = np.exp(-axl) * _horner(_K0B, 2.0 / axl) / np.sqrt(axl)
    out = np.where(small, s_s, s_l)
    return np.where(ax > 0, out, 1.0e20)


def vzatom(Z, r, fparams):
    """Projected atomic potential in V*Angstrom (slicelib.cpp:2666-2716)."""
    r = np.maximum(np.abs(np.asarray(r, dtype=np.float64)), 1.0e-10)
    p = fparams[Z]
    x = 2.0 * PI_K * r
    suml = (p[0] * bessk0(x * np.sqrt(p[1])) + p[2] * bessk0(x * np.sqrt(p[3]))
            + p[4] * bessk0(x * np.sqrt(p[5])))
    x = (PI_K * r) ** 2
    sumg = (p[6] * np.exp(-x / p[7]) / p[7] + p[8] * np.exp(-x / p[9]) / p[9]
            + p[10] * np.exp(-x / p[11]) / p[11])
    return AL * suml + AG * sumg


def slice_index(z, cz_total, nslice):
    """Slice bin of each atom: floor(z/dz), -1 if outside [0, cz) (ModelPotential.cu:63-71)."""
    dz = cz_total / nslice
    kz = np.floor(np.asarray(z, dtype=np.float64) / dz).astype(np.int64)
    bad = (np.asarray(z) < 0.0) | (kz < 0) | (kz >= nslice)
    return np.where(bad, -1, kz)


def potential(x, y, z, Znum, fparams, ax, by, cz_total, nx, ny, nslice, radius):
    """V_z per slice, float64 [nslice, nx, ny] (ModelPotential.cu:27-99, :154-203)."""
    if 2.0 * radius >= ax or 2.0 * radius >= by:
        raise ValueError("cutoff radius must be below half the cell")
    out = np.zeros((nslice, nx, ny), dtype=np.float64)
    kz = slice_index(z, cz_total, nslice)
    dxp, dyp = ax / nx, by / ny
    ixs = np.arange(nx)
    iys = np.arange(ny)
    for a in range(len(x)):
        if kz[a] < 0:
            continue
        xa = x[a] - ax * np.floor(x[a] / ax)
        ya = y[a] - by * np.floor(y[a] / by)
        ddx = np.abs(xa - ixs * dxp)
        ddx = np.where(ddx >= ax / 2.0, ax - ddx, ddx)
        ddy = np.abs(ya - iys * dyp)
        ddy = np.where(ddy >= by / 2.0, by - ddy, ddy)
        sx = np.nonzero(ddx < radius)[0]
        sy = np.nonzero(ddy < radius)[0]
        r = np.sqrt(ddx[sx, None] ** 2 + ddy[None, sy] ** 2)
        m = r < radius
        v = np.where(m, vzatom(int(Znum[a]), np.maximum(r, 1.0e-10), fparams), 0.0)
        out[kz[a]][np.ix_(sx, sy)] += v
    return out


# ------------------------------------------------------------ FFT conventions
def _fft_mod():
    return _sfft if _sfft is not None else np.fft


def kfft(w, workers=1):
    """Kirkland fft: exp(+i..), unscaled, over the last two axes."""
    m = _fft_mod()
    if m is np.fft:
        return np.fft.ifft2(w, axes=(-2, -1), norm="forward")
    return m.ifft2(w, axes=(-2, -1), norm="forward", workers=workers)


def kifft(w, workers=1):
    """Kirkland ifft: exp(-i..), scaled by 1/(nx*ny), over the last two axes."""
    m = _fft_mod()
    if m is np.fft:
        return np.fft.fft2(w, axes=(-2, -1), norm="forward")
    return m.fft2(w, axes=(-2, -1), norm="forward", workers=workers)


# --------------------------------------------------------------- k-space grid
def freqn(n, a):
    """Spatial frequencies k and k^2 as float32 (slicelib.cpp:433-463)."""
    f32 = np.float32
    imid = int(n / 2.0 + 0.5)
    i = np.arange(n)
    num = np.where(i > imid, i - n, i).astype(f32)
    k = num / f32(a)
    return k.astype(f32), (k * k).astype(f32)


def k2max_f32(nx, ny, ax, by, bw=2.0 / 3.0):
    """Squared band limit in float32 (mulslice.cpp:481-489)."""
    f32 = np.float32
    k = f32(nx) / (f32(2.0) * f32(ax))
    t = f32(ny) / (f32(2.0) * f32(by))
    if t < k:
        k = t
    k = f32(bw) * k
    return f32(k * k)


def band_mask(nx, ny, ax, by, bw=2.0 / 3.0):
    kx, kx2 = freqn(nx, ax)
    ky, ky2 = freqn(ny, by)
    return (kx2[:, None] + ky2[None, :]) < k2max_f32(nx, ny, ax, by, bw)


# ------------------------------------------------------------ transmission
def transmission(vz, v0, ax, by, dtype=np.complex64, bw=2.0 / 3.0):
    """Band-limited exp(i sigma V_z) per layer (mulslice.cpp:414-421, :515-522)."""
    nl, nx, ny = vz.shape
    sig = sigma(v0) / 1000.0
    if dtype == np.complex64:
        f32 = np.float32
        wl = f32(wavelength(v0))
        mm0 = f32(1.0) + f32(v0) / f32(511.0)
        vfile = (sig * vz / (float(wl) * float(mm0))).astype(f32)
        ph = (wl * mm0) * vfile
        t = (np.cos(ph.astype(np.float64)).astype(f32)
             + 1j * np.sin(ph.astype(np.float64)).astype(f32)).astype(np.complex64)
    else:
        ph = sig * vz
        t = np.exp(1j * ph).astype(np.complex128)
    m = band_mask(nx, ny, ax, by, bw)
    T = kfft(t)
    T = np.where(m[None], T, 0)
    return kifft(T).astype(dtype)


def propagator_tables(nx, ny, ax, by, v0, dz, ctilt=(0.0, 0.0), precision="f32"):
    """px, py complex tables for one slice thickness (mulslice.cpp:494-513).

    precision "f32" builds the argument in float as mulslice.cpp does;
    "f64" builds it in double (the FP64 oracle and the product's tables)."""
    f32 = np.float32
    kx, kx2 = freqn(nx, ax)
    ky, ky2 = freqn(ny, by)
    if precision == "f32":
        wl = f32(wavelength(v0))
        sc = f32(f32(4.0 * np.arctan(1.0)) * f32(dz))
        tctx = f32(2.0 * np.tan(ctilt[0]))
        tcty = f32(2.0 * np.tan(ctilt[1]))
        tx = (sc * (kx2 * wl - kx * tctx)).astype(np.float64)
        ty = (sc * (ky2 * wl - ky * tcty)).astype(np.float64)
        px = np.cos(tx).astype(f32) + 1j * (-np.sin(tx)).astype(f32)
        py = np.cos(ty).astype(f32) + 1j * (-np.sin(ty)).astype(f32)
        return px.astype(np.complex64), py.astype(np.complex64)
    wl = wavelength(v0)
    kxd, kyd = kx.astype(np.float64), ky.astype(np.float64)
    tx = np.pi * dz * (kxd * kxd * wl - kxd * 2.0 * np.tan(ctilt[0]))
    ty = np.pi * dz * (kyd * kyd * wl - kyd * 2.0 * np.tan(ctilt[1]))
    return np.exp(-1j * tx), np.exp(-1j * ty)


# --------------------------------------------------------------- slice loop
def propagate(W, px, py, mask):
    """Multiply by py(ky) then px(kx), zero outside the band (slicelib.cpp:744-790)."""
    W = W * py[None, :]
    W = W * px[:, None]
    return np.where(mask, W, 0).astype(W.dtype)


def multislice(wave, trans, props, layer_seq, mask, workers=1, detect=None):
    """Run the coherent slice loop on wave [..., nx, ny] (mulslice.cpp:706-739).

    trans [nlayer, nx, ny]; props: list of (px, py) per layer; detect: optional
    (checkpoints, fn) where fn(W) -> array is called after the propagator of each
    checkpoint slice.  Returns the exit wave (and the detector results)."""
    w = np.array(wave, copy=True)
    out = []
    cps = list(detect[0]) if detect else []
    last = cps[-1] if cps else None
    for s, l in enumerate(layer_seq):
        w = w * trans[l]
        W = kfft(w, workers)
        px, py = props[l]
        W = propagate(W, px, py, mask)
        if detect and s in cps:
            out.append(detect[1](W))
            if s == last:
                return w, out
        w = kifft(W, workers).astype(wave.dtype)
    return w, out


# --------------------------------------------------------------------- STEM
def signed_index(n):
    i = np.arange(n)
    return np.where(i < n // 2, i, i - n)


def k_tables_f64(nx, ny, ax, by):
    """C#-style reciprocal coordinates (double) of MSProject.cs:470-484."""
    return signed_index(nx) / ax, signed_index(ny) / by


def probe(nx, ny, ax, by, v0, kap_in, kap_out, df, cs, xy, dtype=np.complex64):
    """Converged probe(s) in real space, [nprobe, nx, ny] (MSProject.cs:458-514)."""
    lam = wavelength(v0)
    kxd, kyd = k_tables_f64(nx, ny, ax, by)
    s = kxd[:, None] ** 2 + kyd[None, :] ** 2
    ap = (s >= kap_in ** 2) & (s <= kap_out ** 2)
    chi = np.pi * (lam * df * s + 0.5 * cs * lam ** 3 * s * s)
    i = signed_index(nx)[:, None]
    j = signed_index(ny)[None, :]
    xy = np.atleast_2d(np.asarray(xy, dtype=np.float64))
    out = np.empty((len(xy), nx, ny), dtype=dtype)
    for p, (xp, yp) in enumerate(xy):
        ph = 2.0 * np.pi * (i * (xp / ax) + j * (yp / by)) - chi
        if dtype == np.complex64:
            P = np.where(ap, np.cos(ph).astype(np.float32) + 1j * np.sin(ph).astype(np.float32), 0)
        else:
            P = np.where(ap, np.exp(1j * ph), 0)
        out[p] = kifft(P.astype(dtype))
    return out


def detector_masks(nx, ny, ax, by, det_k):
    """Boolean annulus masks [ndet, nx, ny]: kin^2 <= s <= kout^2 (MSProject.cs:806-829)."""
    kxd, kyd = k_tables_f64(nx, ny, ax, by)
    s = kxd[:, None] ** 2 + kyd[None, :] ** 2
    return np.stack([(s <= ko * ko) & (s >= ki * ki) for ki, ko in det_k])


def stem(trans, props, layer_seq, mask, probes, det_masks, checkpoints, workers=1):
    """Detector sums [nprobe, ncheck, ndet] in the C# scale (unscaled |Psi(k)|^2)."""
    dm = det_masks.astype(np.float64)

    def fn(W):
        I = (W.real.astype(np.float64) ** 2 + W.imag.astype(np.float64) ** 2)
        return np.einsum("...xy,dxy->...d", I, dm)

    _, res = multislice(probes, trans, props, layer_seq, mask, workers,
                        detect=(list(checkpoints), fn))
    return np.stack(res, axis=-2)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


# ------------------------------------------------------------ CTEM imaging
def ctf(nx, ny, ax, by, v0, cs, df, k_obj, dtype=np.complex128, astig=(0.0, 0.0, 0.0, 0.0)):
    """exp(-i chi) inside the objective aperture (mulslice.cpp:556-633); chi in FP64,
    with 2- and 3-fold astigmatism (dfa2, dfa2phi, dfa3, dfa3phi)."""
    kx, kx2 = freqn(nx, ax)
    ky, ky2 = freqn(ny, by)
    k2 = (kx2[:, None] + ky2[None, :]).astype(np.float32)
    kob = np.float32(k_obj)
    inside = k2 <= np.float32(kob * kob)
    q = k2.astype(np.float64)
    lam = wavelength(v0)
    phi = np.arctan2(ky.astype(np.float64)[None, :], kx.astype(np.float64)[:, None])
    c = chi(q, phi, lam, cs, df, astig)
    return np.where(inside, np.exp(-1j * c), 0).astype(dtype)


def chi(k2, phi, lam, cs, df, astig=(0.0, 0.0, 0.0, 0.0)):
    """Aberration phase of mulslice.cpp:613-619 at |k|^2 = k2 and azimuth phi:
    pi lam k2 (cs lam^2 k2 / 2 - df + dfa2 sin(2(phi - dfa2phi))
    + (2/3) dfa3 lam |k| sin(3(phi - dfa3phi)))."""
    dfa2, dfa2phi, dfa3, dfa3phi = astig
    w = 0.5 * cs * lam * lam * k2 - df
    if dfa2 != 0.0 or dfa3 != 0.0:
        w = w + dfa2 * np.sin(2.0 * (phi - dfa2phi)) + 2.0 * dfa3 * lam * np.sqrt(k2) * np.sin(3.0 * (phi - dfa3phi)) / 3.0
    return np.pi * lam * k2 * w


def defocus_weights(df, df_spread, df_step):
    if df_spread <= 0:
        return np.array([df]), np.array([1.0])
    ndf = int((2.5 * df_spread) / df_step)
    j = np.arange(-ndf, ndf + 1)
    w = np.exp(-0.5 * (j * df_step / df_spread) ** 2)
    return df + j * df_step, w / w.sum()


def ctem_image(exit_wave, ax, by, v0, cs, df, k_obj, df_spread=0.0, df_step=0.0,
               astig=(0.0, 0.0, 0.0, 0.0)):
    """Defocus-averaged image intensity of exit wave(s) [..., nx, ny] (summed over the batch)."""
    nx, ny = exit_wave.shape[-2:]
    W = kfft(exit_wave.astype(np.complex128))
    img = np.zeros((nx, ny))
    for d, w in zip(*defocus_weights(df, df_spread, df_step)):
        psi = kifft(W * ctf(nx, ny, ax, by, v0, cs, d, k_obj, astig=astig))
        I = np.abs(psi) ** 2
        img += w * (I.sum(axis=0) if I.ndim == 3 else I)
    return img


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
    return x ^ (x >> np.uint64(31))


def phonon_displacements(seed, config, natom, sigma):
    """The library's frozen-phonon displacement stream (splitmix64 + Box-Muller)."""
    with np.errstate(over="ignore"):
        i = np.arange(natom, dtype=np.uint64)[:, None]
        k = np.arange(4, dtype=np.uint64)[None, :]
        key = (np.uint64(config) << np.uint64(40)) | (i << np.uint64(2)) | k
        h = _splitmix64(np.uint64(seed) ^ _splitmix64(key))
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    r0 = np.sqrt(-2.0 * np.log(1.0 - u[:, 0]))
    r1 = np.sqrt(-2.0 * np.log(1.0 - u[:, 2]))
    t = 2.0 * np.pi
    return sigma * np.stack([r0 * np.cos(t * u[:, 1]), r0 * np.sin(t * u[:, 1]),
                             r1 * np.cos(t * u[:, 3])], axis=1)


# ------------------------------------------------- Muslib entry points (C#)
def cs_lambda(E):
    """C#/Muslib wavelength, E in volts (Propagator.cpp:17)."""
    return 0.387818 / np.sqrt(E / 1000.0 * (1.0 + 0.978459e-3 * E / 1000))


def muslib_propagator(a, b, gam, thickness, E, tx, ty, N, M):
    """CreatePropagator (Propagator.cpp:5-53) as complex128 [M, N] (row j, column i)."""
    A, B = 1.0 / (a * np.sin(gam)), 1.0 / (b * np.sin(gam))
    GK = np.pi * cs_lambda(E) * thickness
    smax = min(N * 0.5 / a, M * 0.5 / b) ** 2
    i = np.where(np.arange(N) < N // 2, np.arange(N), np.arange(N) - N)
    j = np.where(np.arange(M) < M // 2, np.arange(M), np.arange(M) - M)
    x = i[None, :] * A
    y = j[:, None] * B
    s = x * (x - 2.0 * y * np.cos(gam)) + y * y
    con = GK * s - 2 * np.pi * thickness * np.tan(tx) * x - 2 * np.pi * thickness * np.tan(ty) * y
    return np.where(s >= smax, 0, np.exp(1j * con))


def doyle_turner():
    """Doyle & Turner (1968) table of the Muslib bank (Curves.cpp:86-179), [93, 8]."""
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "multislice_gb300", "data", "doyle_turner.npy")
    return np.load(path)


def dt_rec(z, s, tab=None):
    """Curves.cpp:3-10: sum_j a_j exp(-b_j s^2)."""
    tab = doyle_turner() if tab is None else tab
    s = np.asarray(s, np.float64) * s
    return sum(tab[z, 2 * j] * np.exp(-tab[z, 2 * j + 1] * s) for j in range(4))


def dt_rs2(z, r2, dw, tab=None):
    """Curves.cpp:23-32: 4 pi sum_{b_j>0} a_j/(b_j+dw) exp(-4 pi^2 r2/(b_j+dw))."""
    tab = doyle_turner() if tab is None else tab
    r2 = np.asarray(r2, np.float64) * (-4.0 * np.pi * np.pi)
    sf = np.zeros_like(r2)
    for j in range(4):
        bj = tab[z, 2 * j + 1]
        if bj > 0:
            sf = sf + tab[z, 2 * j] / (bj + dw) * np.exp(r2 / (bj + dw))
    return sf * 4 * np.pi


def dt_rs(z, s, dw, tab=None):
    """Curves.cpp:12-21: the same at radius s."""
    s = np.asarray(s, np.float64)
    return dt_rs2(z, s * s, dw, tab)


def create_pots(types, DW, npoints, dds, vol=None):
    """CreatePots_rec_DT_DW (vol given, Curves.cpp:45-61) or CreatePots_rs_DT_DW
    (Curves.cpp:63-81); the sample points accumulate s += dds as there."""
    s = np.empty(npoints)
    acc = 0.0
    for i in range(npoints):
        s[i] = acc
        acc += dds
    out = np.empty((len(types), npoints))
    for nt, (ty, dw) in enumerate(zip(types, DW)):
        if vol is None:
            out[nt] = dt_rs(ty, s, dw)
        else:
            out[nt] = dt_rec(ty, s) * np.exp(-dw * s * s) * vol
    return out


def _umin(v, n):
    """min(long, ULONG) of the Windows build: an unsigned compare."""
    return v if 0 <= v < n else n


def _rs_rects(k, a, b, atrad, N, M, xx, yy, sg, source, angstrom, periodic, whole):
    """Pixel rectangles (ib, ie, jb, je, x0, y0) of atom k, bounds formula by
    formula as each variant of PG_RS.cpp / Pot_RS.cpp writes them."""
    xk, yk = float(xx[k]), float(yy[k])
    X, Y = (xk, yk) if angstrom else (xk * a, yk * b)
    if whole:
        return [(0, N, 0, M, X, Y)]
    drax = atrad * sg if angstrom else atrad * sg / a
    dray = atrad * sg if angstrom else atrad * sg / b
    if not periodic:
        if not angstrom:                              # PG_RS.cpp:81-84
            r = (max(int((xk - drax) * N), 0), _umin(int((xk + drax) * N), N),
                 max(int((yk - dray) * M), 0), _umin(int((yk + dray) * M), M))
        elif source == "curve":                       # PG_RS.cpp:149-152
            t = lambda v: int(v) if v > 0 else 0
            r = (t(int((xk - drax) * N) / a), t(min(int((xk + drax) * N) / a, N)),
                 t(int((yk - dray) * M) / b), t(min(int((yk + dray) * M) / b, M)))
        else:                                         # PG_RS.cpp:269-272
            r = (max(int((xk - drax) * N / a), 0), _umin(int((xk + drax) * N / a), N),
                 max(int((yk - dray) * M / b), 0), _umin(int((yk + dray) * M / b), M))
        return [r + (X, Y)]
    if not angstrom:                                  # PG_RS.cpp:327-330
        ibb, iee = int((xk - drax) * N), int((xk + drax) * N)
        jbb, jee = int((yk - dray) * M), int((yk + dray) * M)
    else:                                             # PG_RS.cpp:625-628
        ibb, iee = int((xk - drax) / a * N), int((xk + drax) / a * N)
        jbb, jee = int((yk - dray) / b * M), int((yk + dray) / b * M)
    ib0, ie0, jb0, je0 = max(ibb, 0), _umin(iee, N), max(jbb, 0), _umin(jee, M)
    rects = [(ib0, ie0, jb0, je0, X, Y)]          # the nine cases of PG_RS.cpp:337-417
    if jbb < 0:
        rects.append((ib0, ie0, jbb + M, M, X, Y + b))
    if jee >= M:
        rects.append((ib0, ie0, 0, jee - M + 1, X, Y - b))
    if ibb < 0:
        rects.append((ibb + N, N, jb0, je0, X + a, Y))
    if iee >= N:
        rects.append((0, iee - N + 1, jb0, je0, X - a, Y))
    if ibb < 0 and jbb < 0:
        rects.append((ibb + N, N, jbb + M, M, X + a, Y + b))
    if iee >= N and jee >= M:
        rects.append((0, iee - N + 1, 0, jee - M + 1, X - a, Y - b))
    if iee >= N and jbb < 0:
        rects.append((0, iee - N + 1, jbb + M, M, X - a, Y + b))
    if ibb < 0 and jee >= M:
        rects.append((ibb + N, N, 0, jee - M + 1, X + a, Y - b))
    return rects


def muslib_rs_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves=None, dds=None, dw=None,
                   source="curve", angstrom=False, periodic=True, whole=False):
    """(A, B) = (sum res occ, sum res occ ads) per pixel [M, N] of the real-space
    Muslib forms (PG_RS.cpp, Pot_RS.cpp).  source: "curve" (the type's curve at
    r/dds, nothing beyond it), "DT_DW" (Doyle-Turner at r^2 with dw[k]) or
    "DT_TV" (no Debye-Waller term); angstrom: "TV" coordinates."""
    sg, cg = np.sin(gam), np.cos(gam)
    dxa, dyb = a / N, b / M
    tab = doyle_turner() if source != "curve" else None
    A = np.zeros((M, N))
    B = np.zeros((M, N))
    for k in range(len(xx)):
        for ib, ie, jb, je, x0, y0 in _rs_rects(k, a, b, atrad, N, M, xx, yy, sg, source, angstrom,
                                                periodic, whole):
            ib, jb, ie, je = max(ib, 0), max(jb, 0), min(ie, N), min(je, M)
            if ie <= ib or je <= jb:
                continue
            x = np.arange(ib, ie)[None, :] * dxa - x0
            y = np.arange(jb, je)[:, None] * dyb - y0
            r2 = x * (x + 2 * y * cg) + y * y
            if source == "curve":
                npts = curves.shape[1]
                cur = curves[typ[k]]
                ar2 = np.sqrt(r2) / dds
                fl = np.floor(ar2)
                ok = fl < npts - 1
                jjj = np.where(ok, fl, 0).astype(np.int64)
                res = cur[jjj] + (cur[np.minimum(jjj + 1, npts - 1)] - cur[jjj]) * (ar2 - jjj)
                res = np.where(ok, res, 0.0)
            else:
                res = dt_rs2(int(typ[k]), r2, float(dw[k]) if source == "DT_DW" else 0.0, tab)
            A[jb:je, ib:ie] += res * occ[k]
            B[jb:je, ib:ie] += res * occ[k] * ads[k]
    return A, B


def muslib_pg(A, B, E, K=None):
    """Phase grating exp(-K B) exp(-i K A) of PG_RS.cpp:433-441 (K from E volts)."""
    if K is None:
        lam = cs_lambda(E)
        K = lam * np.sqrt(1.0 + (0.0242621 / lam) ** 2)
    return np.exp(-K * B) * np.exp(-1j * K * A)


def muslib_pg_periodic(a, b, gam, E, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic=True):
    """Multiplicative phase grating of PG_rs_curve_DW_periodic (PG_RS.cpp:304-446)
    or, periodic=False, PG_rs_curve_DW_cutpot (:57-119); complex128 [M, N]."""
    A, B = muslib_curve_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic)
    return muslib_pg(A, B, E)


def muslib_curve_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic=True):
    """(sum res occ, sum res occ ads) of the curve forms in fractional coordinates."""
    return muslib_rs_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves=curves, dds=dds,
                          periodic=periodic)


def muslib_rec_potential(a, b, gam, Nmult, Mmult, N, M, SL, EL, xx, yy, ads, occ, typ, DW=None,
                         curves=None, dds=None):
    """Coefficients Potential_rec_DT_DW (Pot_rec_DT_DW.cpp:3-134, DW given) or
    Potential_rec_curve_DW (Pot_rec_curve_DW.cpp:7-164, curves given) add to the
    rows [SL, EL) of an M x N grid; complex128 [EL - SL, N].  Follows the
    reference's loops: row 0, then rows j Mmult < M/2 with their mirrors."""
    cos_gam = -np.cos(gam)
    A_, B_ = 1.0 / (a * np.sin(gam)), 1.0 / (b * np.sin(gam))
    vol = 1.0 / (a * b * np.sin(gam))
    out = np.zeros((EL - SL, N), np.complex128)
    tab = doyle_turner() if curves is None else None
    ds = 1.0 / dds if curves is not None else 0.0
    npts = curves.shape[1] if curves is not None else 0
    ii = np.arange(1, N)
    ii = ii[ii * Nmult < N // 2]
    x = ii * A_
    cols, mcols = ii * Nmult, N - ii * Nmult

    def lookup(k, t):
        """curve value at index position t (array) and the in-range mask."""
        t = np.asarray(t, np.float64)
        fl = np.floor(t)
        ok = fl < npts - 1
        jj = np.where(ok, fl, 0).astype(np.int64)
        c = curves[typ[k]]
        return c[jj] + (c[np.minimum(jj + 1, npts - 1)] - c[jj]) * (t - jj), ok

    def dt(k, s, ss):
        return dt_rec(int(typ[k]), s, tab) * np.exp(-DW[k] * ss) * vol * occ[k]

    if SL == 0:
        for k in range(len(xx)):
            if curves is None:
                res0 = dt_rec(int(typ[k]), 0.0, tab) * vol * occ[k]
            else:
                res0 = curves[typ[k], 0] * occ[k]
            out[0, 0] += res0 * (1 + 1j * ads[k])
            if curves is None:
                res, ok = dt(k, x * 0.5, x * x * 0.25), np.ones(len(x), bool)
            else:
                res, ok = lookup(k, x * 0.5 * ds)
                res = res * occ[k]
            ph = np.exp(1j * (-2. * np.pi * xx[k] * ii.astype(np.float64)))
            out[0, cols[ok]] += (res * ph * (1 + 1j * ads[k]))[ok]
            out[0, mcols[ok]] += (res * np.conj(ph) * (1 + 1j * ads[k]))[ok]
    j = 1
    while j * Mmult < M // 2:
        jj = j * Mmult
        isup = SL <= jj < EL
        islow = SL <= M - jj < EL
        if not (isup or islow):
            j += 1
            continue
        y = j * B_
        y_pow2 = y * y
        y_cosgam = y * cos_gam * 2.
        for k in range(len(xx)):
            pj = np.exp(1j * (-2. * np.pi * yy[k] * float(j)))
            if curves is None:
                r0 = dt(k, np.sqrt(y_pow2 * 0.25), y_pow2 * 0.25)
            else:
                r0, ok0 = lookup(k, y * ds * 0.5)
                if not ok0:
                    continue
                r0 = r0 * occ[k]
            if isup:
                out[jj - SL, 0] += r0 * pj * (1 + 1j * ads[k])
            if islow:
                out[M - jj - SL, 0] += r0 * np.conj(pj) * (1 + 1j * ads[k])
            ss = (x * x + y_pow2 + x * y_cosgam) * 0.25
            ss1 = ss - x * y_cosgam * 0.5
            if curves is None:
                res, res1 = dt(k, np.sqrt(ss), ss), dt(k, np.sqrt(ss1), ss1)
                ok = np.ones(len(x), bool)
            else:
                res, ok1 = lookup(k, np.sqrt(ss) * ds)
                res1, ok2 = lookup(k, np.sqrt(ss1) * ds)
                ok = ok1 & ok2
                res, res1 = res * occ[k], res1 * occ[k]
            pi_ = np.exp(1j * (-2. * np.pi * xx[k] * ii.astype(np.float64)))
            f = 1 + 1j * ads[k]
            if isup:
                out[jj - SL, cols[ok]] += (res * pi_ * pj * f)[ok]
                out[jj - SL, mcols[ok]] += (res1 * np.conj(pi_) * pj * f)[ok]
            if islow:
                out[M - jj - SL, cols[ok]] += (res1 * pi_ * np.conj(pj) * f)[ok]
                out[M - jj - SL, mcols[ok]] += (res * np.conj(pi_ * pj) * f)[ok]
        j += 1
    return out


def illumination_angles(nx, ny, ax, by, v0, acmin, acmax):
    """Tilt vectors (qx, qy) of mulslice.cpp:550-570, in float."""
    f32 = np.float32
    wl = f32(wavelength(v0))
    rx, ry = f32(1.0) / f32(ax), f32(1.0) / f32(by)
    fac = f32(acmax)
    nacx = int((fac / (wl * rx)) + f32(1.5))
    nacy = int((fac / (wl * ry)) + f32(1.5))
    q2max = f32(fac / wl) ** 2
    q2min = f32(f32(acmin) / wl) ** 2
    out = []
    for iqy in range(-nacy, nacy + 1):
        qy = f32(iqy) * ry
        for iqx in range(-nacx, nacx + 1):
            qx = f32(iqx) * rx
            q2 = f32(qx * qx + qy * qy)
            if q2 <= q2max and q2 >= q2min:
                out.append((qx, qy))
    return out


def partial_coherence(trans, props, layer_seq, mask, ax, by, v0, cs, df, k_obj, acmin, acmax,
                      df_spread=0.0, df_step=0.0, astig=(0.0, 0.0, 0.0, 0.0)):
    """Kirkland's partial-coherence image (mulslice.cpp:539-676), FP64."""
    nx, ny = trans.shape[-2:]
    f32 = np.float32
    xpos = (np.arange(nx) * ax).astype(f32) / f32(nx - 1)
    ypos = (np.arange(ny) * by).astype(f32) / f32(ny - 1)
    angles = illumination_angles(nx, ny, ax, by, v0, acmin, acmax)
    img = np.zeros((nx, ny))
    for qx, qy in angles:
        s = (f32(qx) * xpos[:, None] + f32(qy) * ypos[None, :]).astype(f32)
        t = 2.0 * float(f32(np.pi)) * s.astype(np.float64)
        w0 = (np.cos(t).astype(f32) + 1j * np.sin(t).astype(f32)).astype(np.complex128)
        w, _ = multislice(w0, trans, props, layer_seq, mask)
        img += ctem_image(w, ax, by, v0, cs, df, k_obj, df_spread, df_step, astig)
    return img / len(angles), len(angles)
