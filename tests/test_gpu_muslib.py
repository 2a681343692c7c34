"""Muslib-shaped exports (CreatePropagator, ApplyPropagator, the PG_rs_curve_DW_*
phase gratings and Potential_rs_curve_DW_* potentials) against the numpy
restatement of Propagator.cpp, PG_RS.cpp and Pot_RS.cpp, through the C ABI with
the reference's argument lists and C#-layout host buffers."""
import ctypes

import numpy as np
import pytest

from multislice_gb300 import _abi
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("gam", [np.pi / 2, 1.9])
def test_create_and_apply_propagator(gam):
    import torch  # noqa: F401  (initialises the CUDA runtime on device 0)
    lib = _abi.load()
    a, b, dz, E, tx, ty, N, M = 12.0, 15.0, 2.5, 200e3, 0.003, -0.002, 128, 96
    gli = np.zeros((M, N, 2), np.float64)
    cpro = ctypes.c_float(-1)
    assert lib.CreatePropagator(a, b, gam, dz, E, tx, ty, N, M, _p(gli), ctypes.byref(cpro)) == 0
    assert cpro.value == 100.0
    ref = O.muslib_propagator(a, b, gam, dz, E, tx, ty, N, M)
    np.testing.assert_allclose(gli[..., 0] + 1j * gli[..., 1], ref, atol=1e-12)
    rng = np.random.default_rng(0)
    w = rng.standard_normal((M, N)) + 1j * rng.standard_normal((M, N))
    buf = np.ascontiguousarray(np.stack([w.real, w.imag], -1))
    assert lib.ApplyPropagator(a, b, gam, dz, E, tx, ty, N, M, _p(buf), ctypes.byref(cpro)) == 0
    np.testing.assert_allclose(buf[..., 0] + 1j * buf[..., 1], w * ref, atol=1e-12)


def _atoms(seed):
    rng = np.random.default_rng(seed)
    a, b, E, atrad, N, M = 10.0, 11.0, 300e3, 2.0, 96, 128
    na, npts, dds = 40, 400, 0.01
    xx = rng.random(na)
    xx[:4] = [0.01, 0.99, 0.5, 0.02]            # atoms whose boxes wrap the cell
    yy = rng.random(na)
    yy[:4] = [0.01, 0.98, 0.995, 0.5]
    ads = rng.random(na) * 0.05
    occ = 0.5 + 0.5 * rng.random(na)
    typ = rng.integers(0, 3, na).astype(np.int32)
    r = np.arange(npts) * dds
    curves = np.ascontiguousarray(np.stack([z * np.exp(-r / 0.4) for z in (1.0, 2.0, 3.5)]))
    return a, b, E, atrad, N, M, na, npts, dds, xx, yy, ads, occ, typ, curves


@pytest.mark.parametrize("periodic", [True, False])
def test_phase_grating(periodic):
    import torch  # noqa: F401
    lib = _abi.load()
    a, b, E, atrad, N, M, na, npts, dds, xx, yy, ads, occ, typ, curves = _atoms(3)
    fn = lib.PG_rs_curve_DW_periodic if periodic else lib.PG_rs_curve_DW_cutpot
    gli = np.zeros((M, N, 2))
    gli[..., 0] = 1.0
    cpro = ctypes.c_float(0)
    rc = fn(a, b, np.pi / 2, E, atrad, N, M, na, _p(xx), _p(yy), _p(ads), _p(occ), _p(typ), _p(curves),
            npts, dds, _p(gli), ctypes.byref(cpro))
    assert rc == 0 and cpro.value == 100.0
    ref = O.muslib_pg_periodic(a, b, np.pi / 2, E, atrad, N, M, xx, yy, ads, occ, typ, curves, dds,
                               periodic=periodic)
    got = gli[..., 0] + 1j * gli[..., 1]
    assert O.rel_l2(got, ref) < 1e-12
    assert np.abs(got).max() <= 1.0 + 1e-12 and np.abs(got).min() < 0.999


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("gam", [np.pi / 2, 1.75])
def test_potential_curve(periodic, gam):
    import torch  # noqa: F401
    lib = _abi.load()
    a, b, E, atrad, N, M, na, npts, dds, xx, yy, ads, occ, typ, curves = _atoms(7)
    fn = lib.Potential_rs_curve_DW_periodic if periodic else lib.Potential_rs_curve_DW_cutpot
    rng = np.random.default_rng(11)
    base = rng.standard_normal((M, N, 2))
    gli = base.copy()
    cpro = ctypes.c_float(0)
    rc = fn(a, b, gam, atrad, N, M, na, _p(xx), _p(yy), _p(ads), _p(occ), _p(typ), _p(curves), npts, dds,
            _p(gli), ctypes.byref(cpro))
    assert rc == 0 and cpro.value == 100.0
    A, B = O.muslib_curve_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic)
    np.testing.assert_allclose(gli[..., 0] - base[..., 0], A, atol=1e-11)
    np.testing.assert_allclose(gli[..., 1] - base[..., 1], B, atol=1e-11)
    assert A.max() > 1.0
