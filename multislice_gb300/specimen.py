"""Seeded specimen generators and scan geometry for the benchmark workloads.

Host logic only (numpy).  Atom lists use Cartesian Angstrom coordinates with z
along the beam, the content a reference .coo file carries once its fractional
coordinates are scaled by the cell (amodel/include/ModelCoo.cpp:20-90).

Every generator takes ``z_offset``: a rigid shift of the whole crystal along z.
Crystals on ideal sites put whole atomic layers exactly on slice boundaries
when the slice thickness divides the period (Si with a/4 slices, SrTiO3 with
a/2, Au with a/2); binning by floor(z/dz) then depends on the last bit of z.
Shifting by half a slice centres every layer in its slice and removes that
ambiguity without changing the specimen.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SI_DIAMOND_BASIS = np.array([
    [0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0],
    [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25],
])
FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
# SrTiO3 perovskite: Sr (0,0,0), Ti (1/2,1/2,1/2), O at the face centres
SRTIO3_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5],
                         [0.0, 0.5, 0.5]])
SRTIO3_Z = np.array([38, 22, 8, 8, 8])


@dataclass
class Specimen:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    Z: np.ndarray
    ax: float
    by: float
    cz: float

    @property
    def natom(self):
        return len(self.x)


def crystal(a, basis, Zs, ncx, ncy, ncz, z_offset=0.0):
    """Tile a cubic cell of side a, basis in fractional coordinates."""
    basis = np.asarray(basis, dtype=np.float64)
    Zs = np.broadcast_to(np.asarray(Zs), (len(basis),))
    i, j, k = np.meshgrid(np.arange(ncx), np.arange(ncy), np.arange(ncz), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    Z = np.tile(Zs, len(cells)).astype(np.int32)
    return Specimen(pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2] + z_offset, Z,
                    ncx * a, ncy * a, ncz * a)


def si_diamond(ncx=5, ncy=5, ncz=20, a=5.431, z_offset=None):
    """Diamond-cubic Si on ideal sites (8 atoms per cell)."""
    if z_offset is None:
        z_offset = a / 8.0  # half of an a/4 slice
    return crystal(a, SI_DIAMOND_BASIS, 14, ncx, ncy, ncz, z_offset)


def srtio3(ncx=8, ncy=8, ncz=50, a=3.905, z_offset=None):
    """SrTiO3 perovskite on ideal sites (5 atoms per cell)."""
    if z_offset is None:
        z_offset = a / 4.0  # half of an a/2 slice
    return crystal(a, SRTIO3_BASIS, SRTIO3_Z, ncx, ncy, ncz, z_offset)


def fcc_au(ncx=16, ncy=16, ncz=40, a=4.078, z_offset=None):
    """fcc Au on ideal sites (4 atoms per cell)."""
    if z_offset is None:
        z_offset = a / 4.0
    return crystal(a, FCC_BASIS, 79, ncx, ncy, ncz, z_offset)


def jitter(spec: Specimen, sigma, rng):
    """Frozen-phonon configuration: iid Gaussian displacement per axis."""
    d = rng.normal(0.0, sigma, size=(spec.natom, 3))
    return Specimen(spec.x + d[:, 0], spec.y + d[:, 1], spec.z + d[:, 2], spec.Z.copy(),
                    spec.ax, spec.by, spec.cz)


def amorphous(box, thickness, density, dmin, Zs, weights, rng):
    """Atoms uniform in a box with a minimum separation (periodic in x and y), Z
    drawn with the given weights: msl_amorphous (dart throwing on a cell grid in
    the library's host code), seeded from rng."""
    import ctypes

    from . import _abi
    lib = _abi.load()
    seed = int(rng.integers(0, 2 ** 63))
    zs = np.ascontiguousarray(Zs, np.int32)
    w = np.ascontiguousarray(weights, np.float64)
    cap = int(round(density * box[0] * box[1] * thickness)) + 1
    xyz = np.empty((cap, 3), np.float64)
    Z = np.empty(cap, np.int32)
    n = ctypes.c_int()
    rc = lib.msl_amorphous(seed, float(box[0]), float(box[1]), float(thickness), float(density), float(dmin),
                           len(zs), zs.ctypes.data, w.ctypes.data, cap, xyz.ctypes.data, Z.ctypes.data,
                           ctypes.byref(n))
    if rc != _abi.MSL_OK:
        raise _abi.MslError(rc, "msl_amorphous failed")
    k = n.value
    return Specimen(xyz[:k, 0].copy(), xyz[:k, 1].copy(), xyz[:k, 2].copy(), Z[:k].copy(), float(box[0]),
                    float(box[1]), float(thickness))


def uneven_jobs(seed, njobs, max_slices=300, max_box=None):
    """Job descriptions of the uneven-batch workload: grid side from
    {256, 384, 512, 768, 1024}, 20..max_slices slices of 1-2 A, an amorphous
    specimen of 0.05 atoms/A^3 with 1.5 A minimum separation and Z from
    {6, 14, 29, 79} (weights 0.4, 0.3, 0.2, 0.1), 80/200/300 kV, plane-wave or
    probe illumination.  The lateral box is 0.1 A per pixel, capped at max_box A.
    Returns dicts with spec, n, nslice, dz, kev and probe (k_ap, x, y) or None;
    everything follows from the seed."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(njobs):
        n = int(rng.choice([256, 384, 512, 768, 1024]))
        nslice = int(rng.integers(20, max(max_slices, 20) + 1))
        dz = float(rng.uniform(1.0, 2.0))
        box = 0.1 * n if max_box is None else min(0.1 * n, float(max_box))
        spec = amorphous((box, box), nslice * dz, 0.05, 1.5, [6, 14, 29, 79], [0.4, 0.3, 0.2, 0.1], rng)
        kev = float(rng.choice([80.0, 200.0, 300.0]))
        probe = None
        if rng.random() < 0.5:
            probe = (float(mrad_to_k(rng.uniform(10.0, 30.0), kev)), float(rng.uniform(0, box)),
                     float(rng.uniform(0, box)))
        out.append(dict(spec=spec, n=n, nslice=nslice, dz=dz, kev=kev, probe=probe))
    return out


def raster(x0, x1, y0, y1, nx, ny):
    """Probe positions of an nx x ny raster over [x0, x1) x [y0, y1), x-major."""
    xs = x0 + (x1 - x0) * np.arange(nx) / nx
    ys = y0 + (y1 - y0) * np.arange(ny) / ny
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel()], axis=1)


def mrad_to_k(mrad, kev):
    """Scattering angle (mrad) to spatial frequency theta/lambda (1/A)."""
    emass, hc = 510.99906, 12.3984244
    lam = hc / np.sqrt(kev * (2.0 * emass + kev))
    return np.asarray(mrad, dtype=np.float64) * 1e-3 / lam


# --------------------------------------------------------------- workloads
def config_si_ctem():
    """Si [001], 5x5x20 cells, 256^2, dz = a/4 (80 slices), 200 kV plane wave."""
    spec = si_diamond()
    return dict(spec=spec, nx=256, ny=256, nslice=80, kev=200.0, radius=5.0)


def config_srtio3_stem(nprobe_side=64):
    """SrTiO3 [001], 8x8x50 cells, 512^2, 100 slices, 200 kV, 25 mrad probe,
    64x64 raster over the central 2x2 cells, HAADF 80-200 mrad, ABF 11-22 mrad."""
    a = 3.905
    spec = srtio3()
    kev = 200.0
    xy = raster(3 * a, 5 * a, 3 * a, 5 * a, nprobe_side, nprobe_side)
    return dict(spec=spec, nx=512, ny=512, nslice=100, kev=kev, radius=5.0,
                k_ap=float(mrad_to_k(25.0, kev)), probe_xy=xy,
                det_k=[(float(mrad_to_k(80.0, kev)), float(mrad_to_k(200.0, kev))),
                       (float(mrad_to_k(11.0, kev)), float(mrad_to_k(22.0, kev)))])


# ------------------------------------------------------------------- .coo
def parse_coo(text):
    """(cell, records) of .coo text via msl_coo_parse; records [natom, 7] =
    x y z (fractional, wrapped) Z dw ads occ."""
    import ctypes
    from . import _abi
    lib = _abi.load()
    raw = text.encode() if isinstance(text, str) else bytes(text)
    cell = _abi.Cell()
    rc = lib.msl_coo_parse(raw, len(raw), ctypes.byref(cell), None, 0)
    if rc != 0:
        raise _abi.MslError(rc, "not a .coo header")
    rec = np.zeros((max(cell.natom, 1), 7), np.float64)
    rc = lib.msl_coo_parse(raw, len(raw), ctypes.byref(cell), ctypes.c_void_p(rec.ctypes.data),
                           cell.natom)
    if rc != 0:
        raise _abi.MslError(rc, "malformed .coo atom records")
    return cell, rec[: cell.natom]


def read_coo(path):
    """Specimen (Cartesian Angstrom, orthogonal cells) from a .coo file."""
    with open(path, "rb") as f:
        cell, rec = parse_coo(f.read())
    if abs(cell.gamma - 90.0) > 1e-9 or abs(cell.alpha - 90.0) > 1e-9 or abs(cell.beta - 90.0) > 1e-9:
        raise ValueError("only orthogonal cells map onto the slice grid")
    return Specimen(rec[:, 0] * cell.a, rec[:, 1] * cell.b, rec[:, 2] * cell.c,
                    rec[:, 3].astype(np.int32), cell.a, cell.b, cell.c)


def write_coo(spec, path, title=None):
    """Write a Specimen as .coo (header line, fractional records x y z Z 0 0 1)."""
    with open(path, "w") as f:
        if title:
            f.write(f"// {title}\n")
        f.write(f"{spec.ax:.10g} {spec.by:.10g} {spec.cz:.10g} 90 90 90 {spec.natom}\n")
        for x, y, z, Z in zip(spec.x / spec.ax, spec.y / spec.by, spec.z / spec.cz, spec.Z):
            f.write(f"{x:.12f} {y:.12f} {z:.12f} {int(Z)} 0 0 1\n")
