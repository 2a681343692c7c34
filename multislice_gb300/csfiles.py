"""The C# STEM driver's output files (Musli console 1.3 (STEM) 2/MSProject.cs).

.wav  (SaveWav, MSProject.cs:522-596): N*M complex doubles, row j (y) major,
      (re, im) interleaved, then a 160-byte ASCII trailer
      "___ a b thickness pi/2 pi/2 gamma E(kV) N M thickness 0", zero padded.
.stem (FlushSTEMfile, MSProject.cs:697-790): one double per beam position, then
      a 160-byte trailer "~~~ dx dy thickness pi/2 pi/2 gamma E(kV) Nscan Mscan
      thickness 0" (dx, dy: extent of the raster in cell fractions).

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


def _trailer(tag, a, b, th, gam, kev, n, m):
    s = (f"{tag} {a:>12.10g} {b:>12.10g} {th:>12.10g} {math.pi / 2:>10.5g} {math.pi / 2:>10.5g} "
         f"{gam:>10.8g} {kev:>10g} {int(n)} {int(m)} {th:>10g} {0:>5d} ")
    raw = s.encode("ascii")[:TRAILER]
    return raw + b"\0" * (TRAILER - len(raw))


def _parse_trailer(raw, tag):
    text = raw.rstrip(b"\0").decode("ascii")
    f = text.split()
    if not f or f[0] != tag:
        raise ValueError("not a trailer of this kind")
    a, b, th, _, _, gam, kev = (float(x) for x in f[1:8])
    n, m = int(f[8]), int(f[9])
    return dict(a=a, b=b, thickness=th, gamma=gam, kev=kev, n=n, m=m)


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
