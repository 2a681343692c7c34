"""MRC image files: the output format of the reference's LMultiSlice
(ImageSimulation/Image/Image.cu:138-160, MRC.cpp/MRC.h: 1024-byte header of
56 words plus ten 80-character labels, then the data).

Layout written here (MRC2014 conventions): little-endian; words 1-3 nx, ny, nz
(columns, rows, sections); word 4 the mode (2 = float32, 4 = complex64);
words 8-10 the sampling mx, my, mz; 11-13 the cell edges in Angstrom; 14-16
the cell angles; 17-19 the axis map (1, 2, 3); 20-22 min, max, mean; 53 the
"MAP " tag; 54 the machine stamp; 55 rms; 56 the label count.  Section k holds
row y of column x at k*ny*nx + y*nx + x, so an x-major array [ix][iy] is
written with the columns running along iy.
"""
from __future__ import annotations

import struct

import numpy as np

MODE_FLOAT32 = 2
MODE_COMPLEX64 = 4


def write_mrc(path, data, cell=(1.0, 1.0, 1.0), labels=()):
    """Write a 2D or 3D float32 or complex64 array (sections first)."""
    a = np.asarray(data)
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3:
        raise ValueError("MRC data must be 2D or 3D")
    if np.iscomplexobj(a):
        a = a.astype(np.complex64)
        mode = MODE_COMPLEX64
        stats = np.abs(a)
    else:
        a = a.astype(np.float32)
        mode = MODE_FLOAT32
        stats = a
    nz, ny_rows, nx_cols = a.shape
    hdr = bytearray(1024)
    struct.pack_into("<4i", hdr, 0, nx_cols, ny_rows, nz, mode)
    struct.pack_into("<3i", hdr, 16, 0, 0, 0)
    struct.pack_into("<3i", hdr, 28, nx_cols, ny_rows, nz)
    struct.pack_into("<6f", hdr, 40, float(cell[0]), float(cell[1]), float(cell[2]), 90.0, 90.0, 90.0)
    struct.pack_into("<3i", hdr, 64, 1, 2, 3)
    struct.pack_into("<3f", hdr, 76, float(stats.min()), float(stats.max()), float(stats.mean()))
    struct.pack_into("<2i", hdr, 88, 0, 0)
    hdr[208:212] = b"MAP "
    hdr[212:216] = bytes([0x44, 0x44, 0x00, 0x00])
    struct.pack_into("<f", hdr, 216, float(stats.std()))
    labels = [str(s)[:80] for s in labels][:10]
    struct.pack_into("<i", hdr, 220, len(labels))
    for i, s in enumerate(labels):
        hdr[224 + 80 * i: 224 + 80 * i + len(s)] = s.encode("ascii", "replace")
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(np.ascontiguousarray(a).tobytes())


def read_mrc(path):
    """(data [nz, ny, nx], header dict) of a mode 2 or 4 MRC file."""
    with open(path, "rb") as f:
        raw = f.read()
    nx, ny, nz, mode = struct.unpack_from("<4i", raw, 0)
    nsym = struct.unpack_from("<i", raw, 92)[0]
    cell = struct.unpack_from("<3f", raw, 40)
    dtype = {MODE_FLOAT32: np.float32, MODE_COMPLEX64: np.complex64}.get(mode)
    if dtype is None:
        raise ValueError(f"unsupported MRC mode {mode}")
    off = 1024 + nsym
    data = np.frombuffer(raw, dtype=dtype, count=nx * ny * nz, offset=off).reshape(nz, ny, nx)
    nlab = struct.unpack_from("<i", raw, 220)[0]
    labels = [raw[224 + 80 * i: 304 + 80 * i].rstrip(b"\0 ").decode("ascii", "replace") for i in range(nlab)]
    return data.copy(), {"mode": mode, "cell": cell, "labels": labels}
