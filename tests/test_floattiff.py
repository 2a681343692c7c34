"""Kirkland floatTIFF files: the writer here reproduces the reference's
floatTIFF::write byte for byte (golden files made by the reference's own code,
tests/golden/make_tiff_golden.py), and each side reads the other's files."""
import ctypes
import os
import re

import numpy as np
import pytest

from multislice_gb300 import floattiff as FT

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
REF_LIB = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libkirkland_ref.so")
CASES = ("real", "complex", "wide")


def _inputs(name):
    z = np.load(os.path.join(GOLD, "tiff_inputs.npz"))
    npix, dx, dy, rmin, rmax, imin, imax = z[f"{name}_meta"]
    return z[f"{name}_img"], z[f"{name}_par"], int(npix), dx, dy, rmin, rmax, imin, imax


@pytest.mark.parametrize("name", CASES)
def test_writer_matches_reference_bytes(name, tmp_path):
    img, par, npix, dx, dy, rmin, rmax, imin, imax = _inputs(name)
    gold = open(os.path.join(GOLD, f"tiff_{name}.tif"), "rb").read()
    stamp = re.search(rb"\d{4}:\d\d:\d\d \d\d:\d\d:\d\d", gold).group(0).decode()
    FT.write_float_tiff(tmp_path / "o.tif", img, npix=npix, params=par, rmin=rmin, rmax=rmax, imin=imin,
                        imax=imax, dx=dx, dy=dy, datetime=stamp)
    assert open(tmp_path / "o.tif", "rb").read() == gold


@pytest.mark.parametrize("name", CASES)
def test_reader_reads_reference_files(name):
    img, par, npix, *_ = _inputs(name)
    back, np_, pb = FT.read_float_tiff(os.path.join(GOLD, f"tiff_{name}.tif"))
    assert np.array_equal(back, img) and np_ == npix
    assert np.array_equal(pb[1:], par[1:]) and pb[0] == npix


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="oracle/_ref not built (needs the reference tree)")
def test_reference_reader_reads_our_files(tmp_path):
    lib = ctypes.CDLL(REF_LIB)
    lib.kref_tiff_read.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
    rng = np.random.default_rng(3)
    psi = (rng.standard_normal((48, 40)) + 1j * rng.standard_normal((48, 40))).astype(np.complex64)
    FT.write_exit_wave(tmp_path / "w.tif", psi, 20.0, 18.0, 200.0, 80, 0.02508)
    out = np.zeros(96 * 40, np.float32)
    nx, ny, npix = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    par = np.zeros(512, np.float32)
    rc = lib.kref_tiff_read(str(tmp_path / "w.tif").encode(), out.ctypes.data, out.size, ctypes.byref(nx),
                            ctypes.byref(ny), ctypes.byref(npix), par.ctypes.data)
    assert rc == 1 and (nx.value, ny.value, npix.value) == (96, 40, 2)
    img = out.reshape(40, 96).T
    assert np.array_equal(img[:48] + 1j * img[48:], psi)
    assert par[FT.P["ENERGY"]] == 200.0 and par[FT.P["NSLICES"]] == 80
    assert par[FT.P["DX"]] == np.float32(np.float32(20.0) / np.float32(48))


def test_kirkland_wave_and_potential_layer_roundtrip(tmp_path):
    rng = np.random.default_rng(4)
    psi = (rng.standard_normal((32, 24)) + 1j * rng.standard_normal((32, 24))).astype(np.complex64)
    FT.write_exit_wave(tmp_path / "w.tif", psi, 16.0, 12.0, 300.0, 40, 0.01969, ctilt=(0.001, 0.0))
    back, par = FT.read_exit_wave(tmp_path / "w.tif")
    assert np.array_equal(back, psi) and par[FT.P["XCTILT"]] == np.float32(0.001)
    assert par[FT.P["RMAX"]] == psi.real.max() and par[FT.P["IMIN"]] == psi.imag.min()
    vz = rng.random((32, 24)).astype(np.float32)
    par = np.zeros(512, np.float32)
    par[FT.P["C"]], par[FT.P["DX"]], par[FT.P["DY"]] = 1.3575, 0.5, 0.5
    FT.write_float_tiff(tmp_path / "v.tif", vz, params=par, dx=0.5, dy=0.5)
    v, ax, by, cz, _ = FT.read_potential_layer(tmp_path / "v.tif")
    assert np.array_equal(v, vz) and (ax, by) == (16.0, 12.0) and cz == np.float32(1.3575)
