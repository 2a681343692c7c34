"""The C# STEM driver's output files (Musli console 1.3 (STEM) 2/MSProject.cs).

.wav  (SaveWav, MSProject.cs:522-596): N*M complex doubles, row j (y) major,
      (re, im) interleaved, then a 160-byte ASCII trailer
      "___ a b thickness pi/2 pi/2 gamma E(kV) N M thickness 0", zero padded.
.stem (FlushSTEMfile, MSProject.cs:697-790): one double per beam position, then
      a 160-byte trailer "~~~ dx dy thickness pi/2 pi/2 gamma E(kV) Nscan Mscan
      thickness 0" (dx, dy: extent of the raster in cell fractions).
.cbed (SaveDiffraction, MSProject.cs:598-696): the diffraction intensity |Psi(k)|^2
      of the spectrum after the propagator at a thickness checkpoint, N*M doubles
      row j major with both axes shifted by half (zero frequency at (N/2, M/2)),
      then a "~~~ a b thickness ..." trailer.
.slice (SaveSlice, MSProjectReuse.cs:527-560): one slice's phase grating, N*M
      complex doubles, then "___ a*Nmult b*Mmult dz pi/2 pi/2 gamma -1 N M
      slice nslices".
.slice_coo (SaveSlices, MSProjectUseOnce.cs:297-400): the atoms of one slice:
      uint32 count, double slice thickness, then x, y, z (relative to the top of
      the slice), DW, ads, occ as doubles and type, type_ as int32, each an array
      of count values.

The C# code works in the complex conjugate of this library's convention and
stores y-major, so a wave psi[ix][iy] of this library is written as
conj(psi).T; intensities are unaffected.  The trailer numbers follow the .NET
formats of the reference ({0,12:g10} and so on) as closely as Python's general
format allows (exponents, when any, are written in Python's style).
"""
from __future__ import annotations

import math

import numpy as np

TRAILER = 160


def _trailer(tag, a, b, th, gam, kev, n, m, f9=None, f10=0):
    f9 = th if f9 is None else f9
    s = (f"{tag} {a:>12.10g} {b:>12.10g} {th:>12.10g} {math.pi / 2:>10.5g} {math.pi / 2:>10.5g} "
         f"{gam:>10.8g} {kev:>10g} {int(n)} {int(m)} {f9:>10g} {int(f10):>5d} ")
    raw = s.encode("ascii")[:TRAILER]
    return raw + b"\0" * (TRAILER - len(raw))


def _parse_trailer(raw, tag):
    text = raw.rstrip(b"\0").decode("ascii")
    f = text.split()
    if not f or f[0] != tag:
        raise ValueError("not a trailer of this kind")
    a, b, th, _, _, gam, kev = (float(x) for x in f[1:8])
    n, m = int(f[8]), int(f[9])
    return dict(a=a, b=b, thickness=th, gamma=gam, kev=kev, n=n, m=m, f9=float(f[10]), f10=int(f[11]))


def write_wav(path, psi, a, b, thickness, kev, gamma=math.pi / 2):
    """Exit wave psi[ix][iy] (this library's convention) as a C# .wav file."""
    psi = np.asarray(psi)
    nx, ny = psi.shape
    data = np.ascontiguousarray(np.conj(psi).T, dtype=np.complex128)  # [j][i]
    with open(path, "wb") as f:
        f.write(data.tobytes())
        f.write(_trailer("___", a, b, thickness, gamma, kev, nx, ny))


def read_wav(path):
    """(psi[ix][iy] in this library's convention, trailer dict) of a C# .wav file."""
    raw = open(path, "rb").read()
    meta = _parse_trailer(raw[-TRAILER:], "___")
    n, m = meta["n"], meta["m"]
    data = np.frombuffer(raw[: n * m * 16], dtype=np.complex128).reshape(m, n)
    return np.conj(data.T).copy(), meta


def write_stem(path, image, extent, thickness, kev, gamma=math.pi / 2):
    """STEM image [n_scan_x][n_scan_y] as a C# .stem file (beam positions in raster order)."""
    img = np.asarray(image, dtype=np.float64)
    nsx, nsy = img.shape
    with open(path, "wb") as f:
        f.write(np.ascontiguousarray(img).tobytes())
        f.write(_trailer("~~~", extent[0], extent[1], thickness, gamma, kev, nsx, nsy))


def read_stem(path):
    raw = open(path, "rb").read()
    meta = _parse_trailer(raw[-TRAILER:], "~~~")
    vals = np.frombuffer(raw[:-TRAILER], dtype=np.float64)
    return vals.reshape(meta["n"], meta["m"]).copy(), meta


def write_cbed(path, spectrum, a, b, thickness, kev, gamma=math.pi / 2):
    """Diffraction pattern of a spectrum Psi[ix][iy] (this library's unscaled
    forward transform of the exit wave; the C# spectrum is its conjugate, so the
    intensities are the same) as a C# .cbed file."""
    inten = np.abs(np.asarray(spectrum)) ** 2
    nx, ny = inten.shape
    out = np.fft.fftshift(inten.T.astype(np.float64))          # [j][i], zero frequency at the centre
    with open(path, "wb") as f:
        f.write(np.ascontiguousarray(out).tobytes())
        f.write(_trailer("~~~", a, b, thickness, gamma, kev, nx, ny))


def read_cbed(path):
    """(intensity [ix][iy] in unshifted FFT order, trailer dict) of a .cbed file."""
    raw = open(path, "rb").read()
    meta = _parse_trailer(raw[-TRAILER:], "~~~")
    n, m = meta["n"], meta["m"]
    data = np.frombuffer(raw[: n * m * 8], dtype=np.float64).reshape(m, n)
    return np.fft.ifftshift(data).T.copy(), meta


def write_slice(path, trans, a, b, dz, islice, nslices, gamma=math.pi / 2, nmult=1, mmult=1):
    """Transmission function t[ix][iy] (this library's convention) as a C# .slice file."""
    t = np.asarray(trans)
    nx, ny = t.shape
    data = np.ascontiguousarray(np.conj(t).T, dtype=np.complex128)
    with open(path, "wb") as f:
        f.write(data.tobytes())
        f.write(_trailer("___", a * nmult, b * mmult, dz, gamma, -1.0, nx, ny, f9=islice, f10=nslices))


def read_slice(path):
    raw = open(path, "rb").read()
    meta = _parse_trailer(raw[-TRAILER:], "___")
    n, m = meta["n"], meta["m"]
    data = np.frombuffer(raw[: n * m * 16], dtype=np.complex128).reshape(m, n)
    return np.conj(data.T).copy(), meta


SLICE_COO_FIELDS = ("x", "y", "z", "DW", "ads", "occ")


def write_slice_coo(path, thickness, atoms):
    """Atoms of one slice (a dict of equal-length arrays: x, y, z, DW, ads, occ,
    type, type_) as a .slice_coo file."""
    n = len(atoms["x"])
    with open(path, "wb") as f:
        f.write(np.uint32(n).tobytes())
        f.write(np.float64(thickness).tobytes())
        for k in SLICE_COO_FIELDS:
            f.write(np.asarray(atoms[k], np.float64).tobytes())
        for k in ("type", "type_"):
            f.write(np.asarray(atoms[k], np.int32).tobytes())


def read_slice_coo(path):
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw, np.uint32, 1)[0])
    th = float(np.frombuffer(raw, np.float64, 1, 4)[0])
    if len(raw) != 12 + n * (6 * 8 + 2 * 4):
        raise ValueError("truncated .slice_coo file")
    off = 12
    atoms = {}
    for k in SLICE_COO_FIELDS:
        atoms[k] = np.frombuffer(raw, np.float64, n, off).copy()
        off += 8 * n
    for k in ("type", "type_"):
        atoms[k] = np.frombuffer(raw, np.int32, n, off).copy()
        off += 4 * n
    return th, atoms
