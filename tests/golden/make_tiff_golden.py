"""Golden floatTIFF files written by the reference's own writer.

Builds oracle/_ref (oracle/ref/Makefile, which compiles Kirkland's
floatTIFF.cpp unchanged) and writes, with floatTIFF::write
(ImageSimulation/multislice/floatTIFF.cpp:1263-1840):

  tiff_real.tif     64 x 48 real image, square pixels (one strip each)
  tiff_complex.tif  2*40 x 30 complex image (npix 2), rectangular pixels, so
                    the 8-bit preview is stretched
  tiff_wide.tif     1100 x 6 real image: several float strips
  tiff_inputs.npz   the images, parameters and ranges they were written from

Usage: python tests/golden/make_tiff_golden.py [reference root]
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

CASES = {"real": (64, 48, 1, 0.25, 0.25), "complex": (80, 30, 2, 0.3, 0.2), "wide": (1100, 6, 1, 0.1, 0.1)}


def load_ref():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "-j8"],
                   check=True, capture_output=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libkirkland_ref.so"))
    lib.kref_tiff_write.argtypes = ([ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p] + [ctypes.c_float] * 6)
    lib.kref_tiff_read.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
    return lib


def main():
    lib = load_ref()
    rng = np.random.default_rng(17)
    inputs = {}
    for name, (nx, ny, npix, dx, dy) in CASES.items():
        img = rng.standard_normal((nx, ny)).astype(np.float32)
        par = rng.standard_normal(512).astype(np.float32)
        half = nx // npix
        rng_ = [img[:half].min(), img[:half].max()]
        rng_ += [img[half:].min(), img[half:].max()] if npix == 2 else [0.0, 1.0]
        data = np.ascontiguousarray(img.T)
        rc = lib.kref_tiff_write(os.path.join(HERE, f"tiff_{name}.tif").encode(), data.ctypes.data, nx, ny, npix,
                                 par.ctypes.data, *[float(v) for v in rng_], dx, dy)
        assert rc == 1, rc
        inputs[f"{name}_img"] = img
        inputs[f"{name}_par"] = par
        inputs[f"{name}_meta"] = np.array([npix, dx, dy] + [float(v) for v in rng_], np.float64)
    np.savez_compressed(os.path.join(HERE, "tiff_inputs.npz"), **inputs)
    print("wrote", ", ".join(f"tiff_{n}.tif" for n in CASES))


if __name__ == "__main__":
    main()
