"""Kirkland's floating-point TIFF files, the image format of the reference's CPU
multislice programs (ImageSimulation/multislice/floatTIFF.cpp).

A file holds three TIFF images, in this order (floatTIFF.cpp:1263-1840):

1. an 8-bit greyscale preview, stretched by bilinear interpolation to square
   pixels when dx != dy, each half scaled by its own (min, max) when the image
   is complex;
2. the 32-bit IEEE float image itself, rows of nx pixels (a complex image is
   stored side by side, real then imaginary, as one 2*nx wide image, npix = 2);
3. a one-row float "image" of 512 parameters (param[0] = npix; the indices
   are those of slicelib.hpp:118-161, e.g. pDX = 14, pENERGY = 16).

Each image has one 14-entry IFD (strips of about 8 KB, strip offset and count
arrays when there is more than one strip, X/Y resolution rationals; the
parameter IFD carries a 20-character DateTime).  Files are written
little-endian, as the reference writes on little-endian machines; both byte
orders are read.

Arrays here are x-major like the rest of the library: image[ix][iy], with ix
running along a TIFF row.
"""
from __future__ import annotations

import struct
import time

import numpy as np

PMAX = 512
P = dict(NPIX=0, RMAX=1, IMAX=2, RMIN=3, IMIN=4, XBTILT=5, YBTILT=6, C=7, RES=8, XCTILT=9, YCTILT=10,
         DEFOCUS=11, ASTIG=12, THETA=13, DX=14, DY=15, ENERGY=16, OAPERT=17, CS=18, WAVEL=19,
         CAPERT=21, DDF=22, NSLICES=29, MINDET=31, MAXDET=32)

_f32 = np.float32


def _preview(img, npix, rmin, rmax, imin, imax, nx2, ny2):
    """The 8-bit preview: tinter() bilinear interpolation (floatTIFF.cpp:572-600)
    at x = (nx-1) ix/(nx2-1), y = (ny-1) iy/(ny2-1), scaled to 0..255 with the
    float/double mix of the reference (floatTIFF.cpp:1403-1420)."""
    nx, ny = img.shape
    ix2 = np.arange(nx2, dtype=np.float64)
    iy2 = np.arange(ny2, dtype=np.float64)
    x = (nx - 1) * ix2 / (nx2 - 1) if nx2 > 1 else np.zeros(1)
    y = (ny - 1) * iy2 / (ny2 - 1) if ny2 > 1 else np.zeros(1)
    X, Y = np.meshgrid(x, y, indexing="ij")                     # [nx2][ny2]
    ix = np.clip(X.astype(np.int64), 0, max(nx - 2, 0))
    iy = np.clip(Y.astype(np.int64), 0, max(ny - 2, 0))
    ixp = np.minimum(ix + 1, nx - 1)
    iyp = np.minimum(iy + 1, ny - 1)
    f = img.astype(np.float32)
    f00, f01, f10, f11 = f[ix, iy], f[ix, iyp], f[ixp, iy], f[ixp, iyp]
    x1, y1 = ix.astype(np.float32), iy.astype(np.float32)
    d = ((f00 - f01) - f10) + f11
    c = (f01 - f00) - d * x1
    b = (f10 - f00) - d * y1
    a = ((f00 - b * x1) - c * y1) - (d * x1) * y1
    a, b, c, d = (v.astype(np.float64) for v in (a, b, c, d))
    # tinter returns float; write() keeps z in a double, so the scaling is double
    z = (a + b * X + c * Y + d * X * Y).astype(np.float32).astype(np.float64)
    scaler = float(_f32(255.0) / _f32(_f32(rmax) - _f32(rmin)))
    lt = scaler * (z - float(_f32(rmin))) + 0.5
    if npix > 1:
        scalei = float(_f32(255.0) / _f32(_f32(imax) - _f32(imin)))
        li = scalei * (z - float(_f32(imin))) + 0.5
        right = (np.arange(nx2) >= nx2 // npix)[:, None]
        lt = np.where(right, li, lt)
    lv = np.trunc(lt)
    return np.clip(lv, 0, 255).astype(np.uint8)


class _Out:
    def __init__(self):
        self.buf = bytearray(8)

    @property
    def off(self):
        return len(self.buf)

    def put(self, b):
        self.buf += b

    def pad_even(self):
        if len(self.buf) % 2:
            self.buf += b"\0"


def _ifd(tags):
    """14 entries (tag, type, count, value) -> bytes, next-IFD pointer excluded."""
    out = struct.pack("<h", len(tags))
    for tag, typ, cnt, val in tags:
        out += struct.pack("<HHiI", tag, typ, cnt, val & 0xFFFFFFFF)
    return out


def _strips(o, rows, nrows):
    """Write row blocks as strips; return (offset value, count value, nstrips)
    of the StripOffsets / StripByteCounts tags, writing their arrays if needed."""
    offs, counts = [], []
    for r0 in range(0, len(rows), nrows):
        chunk = b"".join(rows[r0:r0 + nrows])
        offs.append(o.off)
        counts.append(len(chunk))
        o.put(chunk)
    n = len(offs)
    if n > 1:
        ov = o.off
        o.put(struct.pack(f"<{n}i", *offs))
        cv = o.off
        o.put(struct.pack(f"<{n}i", *counts))
        return ov, cv, n
    return offs[0], counts[0], 1


def write_float_tiff(path, image, npix=1, params=None, rmin=None, rmax=None, imin=None, imax=None,
                     dx=1.0, dy=None, datetime=None):
    """Write image[ix][iy] (float32; complex images as a 2*nx wide real array with
    npix = 2) in floatTIFF's layout.  rmin..imax scale the 8-bit preview (default:
    the data range of each half); dx, dy are the pixel sizes (floatTIFF::write's
    dxi, dyi).  datetime: 19 characters "YYYY:MM:DD HH:MM:SS" (default: now)."""
    img = np.asarray(image, dtype=np.float32)
    if img.ndim != 2 or npix not in (1, 2):
        raise ValueError("image must be 2D and npix 1 or 2")
    nx, ny = img.shape
    half = nx // npix
    if rmin is None:
        rmin, rmax = float(img[:half].min()), float(img[:half].max())
    if npix == 2 and imin is None:
        imin, imax = float(img[half:].min()), float(img[half:].max())
    imin = 0.0 if imin is None else imin
    imax = 1.0 if imax is None else imax
    if abs(_f32(rmax) - _f32(rmin)) < 1.0e-20:
        raise ValueError("floatTIFF: rmax - rmin is zero")
    par = np.zeros(PMAX, np.float32)
    if params is not None:
        p = np.asarray(params, np.float32).ravel()[:PMAX]
        par[:len(p)] = p
    par[0] = npix
    dxf = _f32(dx if dx is not None else 1.0)
    if dxf <= 0:
        dxf = _f32(1.0)
    dyf = _f32(dy) if dy is not None else dxf
    if dyf <= 0:
        dyf = dxf
    if dxf > dyf:
        nx2, ny2 = int(_f32(_f32(_f32(nx) * dxf) / dyf) + _f32(0.5)), ny
    elif dxf < dyf:
        nx2, ny2 = nx, int(_f32(_f32(_f32(ny) * dyf) / dxf) + _f32(0.5))
    else:
        nx2, ny2 = nx, ny
    o = _Out()
    base = {254: (4, 1, 0), 259: (3, 1, 1), 262: (3, 1, 1), 277: (3, 1, 1), 296: (3, 1, 2)}

    def tags(w, h, bits, nrows, so, sc, ns, xr, yr, fmt, extra=None):
        t = dict(base)
        t.update({256: (4, 1, w), 257: (4, 1, h), 258: (3, 1, bits), 273: (4, ns, so), 278: (4, 1, nrows),
                  279: (4, ns, sc), 282: (5, 1, xr), 283: (5, 1, yr), 339: (3, 1, fmt)})
        if extra:
            t.pop(296)
            t.update(extra)
        return [(k,) + t[k] for k in sorted(t)]

    # 1. 8-bit preview
    pv = _preview(img, npix, rmin, rmax, imin, imax, nx2, ny2)
    nrows = min(max(8192 // nx2, 1), ny2)
    so, sc, ns = _strips(o, [pv[:, iy].tobytes() for iy in range(ny2)], nrows)
    xy = struct.pack("<ii", int(nx2 / 0.04), 100)
    xr = o.off
    o.put(xy)
    yr = o.off
    o.put(xy)
    o.pad_even()
    ifd1 = o.off
    o.put(_ifd(tags(nx2, ny2, 8, nrows, so, sc, ns, xr, yr, 1)))
    p12 = o.off
    o.put(b"\0\0\0\0")
    # 2. float image
    nrows = min(max(8192 // (nx * 4), 1), ny)
    so, sc, ns = _strips(o, [np.ascontiguousarray(img[:, iy]).tobytes() for iy in range(ny)], nrows)
    xr = o.off
    o.put(struct.pack("<ii", int(nx / 0.04), 100))
    yres = int(float(_f32(dyf / dxf)) * float(nx) / 0.04)
    yr = o.off
    o.put(struct.pack("<ii", yres, 100))
    o.pad_even()
    ifd2 = o.off
    o.put(_ifd(tags(nx, ny, 32, nrows, so, sc, ns, xr, yr, 3)))
    p23 = o.off
    o.put(b"\0\0\0\0")
    # 3. parameters, DateTime in place of ResolutionUnit
    po = o.off
    o.put(par.astype("<f4").tobytes())
    xr = o.off
    o.put(struct.pack("<ii", int(nx / 0.04), 100))
    yr = o.off
    o.put(struct.pack("<ii", yres, 100))
    dt = datetime or time.strftime("%Y:%m:%d %H:%M:%S")
    dto = o.off
    o.put(dt.encode("ascii")[:19].ljust(20, b"\0"))
    o.pad_even()
    ifd3 = o.off
    o.put(_ifd(tags(PMAX, 1, 32, 1, po, PMAX * 4, 1, xr, yr, 3, extra={306: (2, 1, dto)})))
    o.put(b"\0\0\0\0")
    buf = o.buf
    buf[0:8] = struct.pack("<2sHI", b"II", 42, ifd1)
    buf[p12:p12 + 4] = struct.pack("<I", ifd2)
    buf[p23:p23 + 4] = struct.pack("<I", ifd3)
    with open(path, "wb") as fh:
        fh.write(bytes(buf))


def _read_ifd(raw, off, e):
    n = struct.unpack_from(e + "H", raw, off)[0]
    tags = {}
    for k in range(n):
        tag, typ, cnt = struct.unpack_from(e + "HHI", raw, off + 2 + 12 * k)
        voff = off + 2 + 12 * k + 8
        size = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8}.get(typ, 4) * cnt
        if typ in (3, 4) and size > 4:
            ptr = struct.unpack_from(e + "I", raw, voff)[0]
            vals = struct.unpack_from(e + ("H" if typ == 3 else "I") * cnt, raw, ptr)
        elif typ == 3:
            vals = struct.unpack_from(e + "H" * cnt, raw, voff)
        elif typ == 4:
            vals = struct.unpack_from(e + "I", raw, voff)
        else:
            vals = struct.unpack_from(e + "I", raw, voff)
        tags[tag] = (typ, cnt, vals)
    nxt = struct.unpack_from(e + "I", raw, off + 2 + 12 * n)[0]
    return tags, nxt


def _strip_bytes(raw, tags):
    offs, counts = tags[273][2], tags[279][2]
    return b"".join(raw[o:o + c] for o, c in zip(offs, counts))


def read_float_tiff(path):
    """(image[ix][iy] float32, npix, params[512] float32) of a floatTIFF file: the
    first 32-bit float image and the parameter row that follows it
    (floatTIFF.cpp:611-671, :731-848)."""
    raw = open(path, "rb").read()
    order = raw[:2]
    if order not in (b"II", b"MM"):
        raise ValueError("not a TIFF file")
    e = "<" if order == b"II" else ">"
    if struct.unpack_from(e + "H", raw, 2)[0] != 42:
        raise ValueError("not a TIFF file")
    off = struct.unpack_from(e + "I", raw, 4)[0]
    tags, nxt = _read_ifd(raw, off, e)
    while not (tags.get(339, (0, 0, (1,)))[2][0] == 3 and tags[258][2][0] == 32):
        if nxt == 0:
            raise ValueError("no floating-point image in the file")
        tags, nxt = _read_ifd(raw, nxt, e)
    w, h = tags[256][2][0], tags[257][2][0]
    data = np.frombuffer(_strip_bytes(raw, tags), dtype=e + "f4", count=w * h).reshape(h, w)
    image = np.ascontiguousarray(data.T.astype(np.float32))
    params = np.zeros(PMAX, np.float32)
    npix = 1
    if nxt:
        ptags, _ = _read_ifd(raw, nxt, e)
        if ptags.get(339, (0, 0, (0,)))[2][0] == 3 and ptags[258][2][0] == 32:
            pb = _strip_bytes(raw, ptags)
            npar = min(len(pb) // 4, PMAX)
            params[:npar] = np.frombuffer(pb, dtype=e + "f4", count=npar)
            npix = int(params[0] + 0.5)
    return image, npix, params


# ---------------------------------------------------------- Kirkland files
def write_exit_wave(path, psi, ax, by, kev, nslices, wavelength, ctilt=(0.0, 0.0), params=None):
    """Exit wave psi[ix][iy] as mulslice writes it (mulslice.cpp:744-786): a
    2*nx wide image, real part then imaginary part, npix = 2, with the range,
    tilt, energy, pixel size, wavelength and slice-count parameters."""
    psi = np.asarray(psi)
    nx, ny = psi.shape
    re, im = psi.real.astype(np.float32), psi.imag.astype(np.float32)
    par = np.zeros(PMAX, np.float32) if params is None else np.asarray(params, np.float32).copy()
    rmin, rmax, imin, imax = re.min(), re.max(), im.min(), im.max()
    dx = _f32(_f32(ax) / _f32(nx))
    dy = _f32(_f32(by) / _f32(ny))
    for k, v in (("RMAX", rmax), ("IMAX", imax), ("RMIN", rmin), ("IMIN", imin), ("XCTILT", ctilt[0]),
                 ("YCTILT", ctilt[1]), ("ENERGY", kev), ("DX", dx), ("DY", dy), ("WAVEL", wavelength),
                 ("NSLICES", nslices)):
        par[P[k]] = v
    write_float_tiff(path, np.concatenate([re, im], axis=0), npix=2, params=par, rmin=rmin, rmax=rmax,
                     imin=imin, imax=imax, dx=dx, dy=dy)


def read_exit_wave(path):
    """(psi[ix][iy] complex64, params) of a complex floatTIFF file."""
    img, npix, par = read_float_tiff(path)
    if npix != 2:
        raise ValueError("not a complex image")
    nx = img.shape[0] // 2
    return (img[:nx] + 1j * img[nx:]).astype(np.complex64), par


def write_image(path, pix, ax, by, kev, wavelength, lens=None, params=None):
    """Real image pix[ix][iy] (npix = 1), with the lens parameters of
    mulslice.cpp:761-773 when given (df, aobj, cs, acmax, ddf)."""
    pix = np.asarray(pix, np.float32)
    nx, ny = pix.shape
    par = np.zeros(PMAX, np.float32) if params is None else np.asarray(params, np.float32).copy()
    rmin, rmax = pix.min(), pix.max()
    dx = _f32(_f32(ax) / _f32(nx))
    dy = _f32(_f32(by) / _f32(ny))
    for k, v in (("RMAX", rmax), ("RMIN", rmin), ("ENERGY", kev), ("DX", dx), ("DY", dy), ("WAVEL", wavelength)):
        par[P[k]] = v
    if lens:
        for k in ("DEFOCUS", "OAPERT", "CS", "CAPERT", "DDF"):
            if k.lower() in lens:
                par[P[k]] = lens[k.lower()]
    write_float_tiff(path, pix, npix=1, params=par, rmin=rmin, rmax=rmax, dx=dx, dy=dy)


def read_potential_layer(path):
    """A projected-potential layer as mulslice reads it (mulslice.cpp:360-420):
    (vz[ix][iy], ax = pDX nx, by = pDY ny, cz = pC, params).  mulslice turns it
    into exp(i lambda mm0 vz)."""
    img, npix, par = read_float_tiff(path)
    if npix != 1:
        raise ValueError("potential layer must be a real image")
    nx, ny = img.shape
    return img, float(par[P["DX"]]) * nx, float(par[P["DY"]]) * ny, float(par[P["C"]]), par
