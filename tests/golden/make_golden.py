"""Generate the golden vectors under tests/golden from the reference's own code.

Runs only where the reference tree exists: it first builds oracle/_ref with
oracle/ref/Makefile (FFTW 2.1.5 float + Kirkland's cfpix.cpp/slicelib.cpp,
compiled unchanged), then calls it through ctypes:

  vzatom.npz       Kirkland vzatom (slicelib.cpp:2666-2716) with FPARAMS.DAT
                   coefficients at a grid of (Z, r); wavelength/sigma values.
  si_small.npz     Si 2x2x2 cells, 64^2, 8 slices: potential (binned real-space
                   sum of vzatom), band-limited transmission, CTEM exit wave of
                   32 slices (mulslice.cpp:706-739) and per-slice intensity.
  si_config1.npz   Si 5x5x20 cells, 256^2, 80 slices, 200 kV: CTEM exit wave.
  stem_small.npz   SrTiO3 2x2x10 cells, 128^2, 20 slices: STEM detector sums of
                   16 probes at two thickness checkpoints.
  stem_config2.npz SrTiO3 8x8x50 cells, 512^2, 100 slices: detector sums of 8
                   probes of the 64x64 raster.

Usage: python tests/golden/make_golden.py [reference root]
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from multislice_gb300 import specimen as S  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
D = ctypes.POINTER(ctypes.c_double)
F = ctypes.POINTER(ctypes.c_float)
I = ctypes.POINTER(ctypes.c_int)


def ptr(a, t):
    return a.ctypes.data_as(t)


def load_ref():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "-j8"],
                   check=True, capture_output=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libkirkland_ref.so"))
    lib.kref_vzatom.restype = ctypes.c_double
    lib.kref_vzatom.argtypes = [ctypes.c_int, ctypes.c_double]
    lib.kref_wavelength.restype = ctypes.c_double
    lib.kref_wavelength.argtypes = [ctypes.c_double]
    lib.kref_sigma.restype = ctypes.c_double
    lib.kref_sigma.argtypes = [ctypes.c_double]
    fp = np.ascontiguousarray(np.load(os.path.join(ROOT, "multislice_gb300", "data", "fparams.npy")))
    assert lib.kref_set_fparams(ptr(fp, D), 104) == 0
    return lib


def potential(lib, spec, nx, ny, nslice, radius):
    out = np.zeros((nslice, nx, ny), np.float64)
    x = np.ascontiguousarray(spec.x, np.float64)
    y = np.ascontiguousarray(spec.y, np.float64)
    z = np.ascontiguousarray(spec.z, np.float64)
    Z = np.ascontiguousarray(spec.Z, np.int32)
    rc = lib.kref_potential(len(x), ptr(x, D), ptr(y, D), ptr(z, D), ptr(Z, I),
                            ctypes.c_double(spec.ax), ctypes.c_double(spec.by),
                            ctypes.c_double(spec.cz), nx, ny, nslice, ctypes.c_double(radius),
                            ptr(out, D))
    assert rc == 0
    return out


def transmission(lib, vz, ax, by, kev, dz):
    nl, nx, ny = vz.shape
    out = np.zeros((nl, nx, ny, 2), np.float32)
    cz = np.full(nl, dz, np.float64)
    vz = np.ascontiguousarray(vz)
    lib.kref_transmission(nx, ny, ctypes.c_double(ax), ctypes.c_double(by), ctypes.c_double(kev),
                          nl, ptr(vz, D), ptr(cz, D), ptr(out, F))
    return out[..., 0] + 1j * out[..., 1]


def ctem(lib, vz, ax, by, kev, dz, seq):
    nl, nx, ny = vz.shape
    cz = np.full(nl, dz, np.float64)
    seq = np.ascontiguousarray(seq, np.int32)
    out = np.zeros((nx, ny, 2), np.float32)
    inten = np.zeros(len(seq), np.float64)
    vz = np.ascontiguousarray(vz)
    lib.kref_ctem(nx, ny, ctypes.c_double(ax), ctypes.c_double(by), ctypes.c_double(kev), nl,
                  ptr(vz, D), ptr(cz, D), len(seq), ptr(seq, I), ctypes.c_double(0.0),
                  ctypes.c_double(0.0), None, ptr(out, F), ptr(inten, D))
    return (out[..., 0] + 1j * out[..., 1]).astype(np.complex64), inten


def stem(lib, vz, ax, by, kev, dz, seq, k_ap, xy, det_k, cps, df=0.0, cs=0.0):
    nl, nx, ny = vz.shape
    cz = np.full(nl, dz, np.float64)
    seq = np.ascontiguousarray(seq, np.int32)
    xy = np.ascontiguousarray(xy, np.float64)
    dk = np.ascontiguousarray(det_k, np.float64)
    cps = np.ascontiguousarray(cps, np.int32)
    out = np.zeros((len(xy), len(cps), len(dk)), np.float64)
    vz = np.ascontiguousarray(vz)
    lib.kref_stem(nx, ny, ctypes.c_double(ax), ctypes.c_double(by), ctypes.c_double(kev), nl,
                  ptr(vz, D), ptr(cz, D), len(seq), ptr(seq, I), ctypes.c_double(0.0),
                  ctypes.c_double(k_ap), ctypes.c_double(df), ctypes.c_double(cs), len(xy),
                  ptr(xy, D), len(dk), ptr(dk, D), len(cps), ptr(cps, I), ptr(out, D))
    return out


def main():
    lib = load_ref()
    # 1. atom form and constants
    Zs = np.array([1, 6, 8, 14, 22, 29, 38, 79, 92], np.int32)
    rs = np.array([1e-12, 1e-6, 0.01, 0.05, 0.1, 0.3, 0.7, 1.0, 1.5, 2.5, 4.0, 6.0], np.float64)
    vz = np.array([[lib.kref_vzatom(int(z), float(r)) for r in rs] for z in Zs])
    kevs = np.array([80.0, 200.0, 300.0])
    np.savez(os.path.join(HERE, "vzatom.npz"), Z=Zs, r=rs, vz=vz, kev=kevs,
             wavelength=np.array([lib.kref_wavelength(k) for k in kevs]),
             sigma=np.array([lib.kref_sigma(k) for k in kevs]))

    # 2. small Si case
    a = 5.431
    spec = S.si_diamond(2, 2, 2, a)
    v = potential(lib, spec, 64, 64, 8, 3.0)
    t = transmission(lib, v, spec.ax, spec.by, 200.0, a / 4)
    seq = np.tile(np.arange(8), 4)
    w, inten = ctem(lib, v, spec.ax, spec.by, 200.0, a / 4, seq)
    np.savez_compressed(os.path.join(HERE, "si_small.npz"), v=v, t=t.astype(np.complex64), seq=seq,
                        wave=w, intensity=inten, ax=spec.ax, by=spec.by, cz=spec.cz, kev=200.0,
                        dz=a / 4, radius=3.0)

    # 3. Si config: 256^2, 80 slices
    cfg = S.config_si_ctem()
    spec = cfg["spec"]
    v = potential(lib, spec, 256, 256, 80, cfg["radius"])
    w, inten = ctem(lib, v, spec.ax, spec.by, 200.0, spec.cz / 80, np.arange(80))
    np.savez_compressed(os.path.join(HERE, "si_config1.npz"), wave=w, intensity=inten,
                        v_checksum=np.array([v.sum(), (v ** 2).sum()]), v0=v[0].astype(np.float32))

    # 4. small STEM case
    a = 3.905
    spec = S.srtio3(2, 2, 10, a)
    kev = 200.0
    v = potential(lib, spec, 128, 128, 20, 3.0)
    xy = S.raster(0.5 * a, 1.5 * a, 0.5 * a, 1.5 * a, 4, 4)
    det_k = np.array([[S.mrad_to_k(80, kev), S.mrad_to_k(200, kev)],
                      [S.mrad_to_k(11, kev), S.mrad_to_k(22, kev)],
                      [0.0, 100.0]])
    k_ap = float(S.mrad_to_k(25.0, kev))
    cps = [9, 19]
    dsum = stem(lib, v, spec.ax, spec.by, kev, a / 2, np.arange(20), k_ap, xy, det_k, cps)
    np.savez_compressed(os.path.join(HERE, "stem_small.npz"), v=v.astype(np.float32), xy=xy,
                        det_k=det_k, k_ap=k_ap, cps=np.array(cps), det=dsum, ax=spec.ax,
                        by=spec.by, kev=kev, dz=a / 2)

    # 5. SrTiO3 config: 512^2, 100 slices, 8 probes of the raster
    cfg = S.config_srtio3_stem()
    spec = cfg["spec"]
    v = potential(lib, spec, 512, 512, 100, cfg["radius"])
    idx = np.array([0, 63, 520, 1111, 2080, 2730, 3333, 4095])
    xy = cfg["probe_xy"][idx]
    dsum = stem(lib, v, spec.ax, spec.by, 200.0, spec.cz / 100, np.arange(100), cfg["k_ap"], xy,
                np.array(cfg["det_k"]), [99])
    np.savez_compressed(os.path.join(HERE, "stem_config2.npz"), idx=idx, xy=xy, det=dsum,
                        v_checksum=np.array([v.sum(), (v ** 2).sum()]))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
