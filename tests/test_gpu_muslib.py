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


def _rs_inputs(src, coord, seed=9):
    rng = np.random.default_rng(seed)
    a, b, E, atrad, N, M, na = 9.0, 10.5, 200e3, 1.8, 80, 96, 30
    xx, yy = rng.random(na), rng.random(na)
    xx[:4] = [0.01, 0.985, 0.5, 0.03]              # boxes that cross the cell edges
    yy[:4] = [0.02, 0.97, 0.995, 0.5]
    if coord == "TV":
        xx, yy = xx * a, yy * b                    # Angstrom coordinates
    ads = rng.random(na) * 0.05
    occ = 0.5 + 0.5 * rng.random(na)
    dw = 0.2 + 0.6 * rng.random(na)
    if src == "curve":
        typ = rng.integers(0, 3, na).astype(np.int32)
        r = np.arange(300) * 0.01
        curves = np.ascontiguousarray(np.stack([z * np.exp(-r / 0.35) for z in (1.0, 2.0, 3.5)]))
    else:
        typ = rng.choice(np.array([8, 22, 38], np.int32), na)
        curves = None
    return a, b, E, atrad, N, M, na, xx, yy, ads, occ, dw, typ, curves


@pytest.mark.parametrize("name", _abi.MUSLIB_RS)
@pytest.mark.parametrize("gam", [np.pi / 2, 1.8])
def test_real_space_forms(name, gam):
    """Every PG_rs_* / Potential_rs_* export against the restatement of its own
    box bounds, radial source and wrap rule."""
    import torch  # noqa: F401
    lib = _abi.load()
    kind, _, src, coord, wrap = name.split("_")
    a, b, E, atrad, N, M, na, xx, yy, ads, occ, dw, typ, curves = _rs_inputs(src, coord)
    rng = np.random.default_rng(1)
    base = rng.standard_normal((M, N, 2))
    gli = base.copy()
    cpro = ctypes.c_float(0)
    head = (a, b, gam, E, atrad) if kind == "PG" else (a, b, gam, atrad)
    common = (N, M, na, _p(xx), _p(yy))
    if src == "curve":
        tail = (_p(ads), _p(occ), _p(typ), _p(curves), curves.shape[1], 0.01, _p(gli), ctypes.byref(cpro))
    elif coord == "DW":
        tail = (_p(dw), _p(ads), _p(occ), _p(typ), _p(gli), ctypes.byref(cpro))
    else:
        tail = (_p(ads), _p(occ), _p(typ), _p(gli), ctypes.byref(cpro))
    assert getattr(lib, name)(*head, *common, *tail) == 0
    source = "curve" if src == "curve" else f"DT_{coord}"
    A, B = O.muslib_rs_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves=curves, dds=0.01,
                            dw=dw, source=source, angstrom=coord == "TV", periodic=wrap == "periodic")
    assert A.max() > 0.5
    got = gli[..., 0] + 1j * gli[..., 1]
    b0 = base[..., 0] + 1j * base[..., 1]
    if kind == "PG":
        assert O.rel_l2(got, b0 * O.muslib_pg(A, B, E)) < 1e-12
    else:
        np.testing.assert_allclose(gli[..., 0] - base[..., 0], A, atol=1e-10)
        np.testing.assert_allclose(gli[..., 1] - base[..., 1], B, atol=1e-10)
    if wrap == "periodic":
        assert cpro.value == 100.0
    else:
        ref = np.float32(0)
        for _ in range(na):
            ref = np.float32(np.float64(ref) + 100.0 / na)
        assert cpro.value == ref


def test_one_atom_grating():
    import torch  # noqa: F401
    lib = _abi.load()
    a, b, gam, K, N, M = 8.0, 8.0, 1.9, 0.025, 64, 64
    r = np.arange(500) * 0.01
    cur = np.ascontiguousarray(4.0 * np.exp(-r / 0.5))
    gli = np.zeros((M, N, 2))
    gli[..., 0] = 1.0
    assert lib.PG_rs_curve_DW_cutpot_oneatom(a, b, gam, K, 1.0, N, M, 0.3, 0.7, 0.04, 0.9, _p(cur), 500,
                                             0.01, _p(gli)) == 0
    A, B = O.muslib_rs_sums(a, b, gam, 1.0, N, M, np.array([0.3]), np.array([0.7]), np.array([0.04]),
                            np.array([0.9]), np.array([0]), curves=cur[None], dds=0.01, periodic=False,
                            whole=True)
    assert O.rel_l2(gli[..., 0] + 1j * gli[..., 1], O.muslib_pg(A, B, 0, K=K)) < 1e-12


@pytest.mark.parametrize("form", ["DT", "curve"])
@pytest.mark.parametrize("gam,mult,band", [(np.pi / 2, (1, 1), (0, 64)), (1.75, (2, 1), (0, 40)),
                                           (np.pi / 2, (1, 3), (10, 60))])
def test_reciprocal_space_potential(form, gam, mult, band):
    import torch  # noqa: F401
    lib = _abi.load()
    rng = np.random.default_rng(21)
    a, b, N, M, na = 11.0, 12.0, 48, 64, 40
    Nmult, Mmult = mult
    SL, EL = band
    xx, yy = rng.random(na), rng.random(na)
    ads, occ = rng.random(na) * 0.05, 0.5 + 0.5 * rng.random(na)
    zs = np.array([8, 22, 38], np.int32)
    pick = rng.integers(0, 3, na)
    dwv = np.array([0.3, 0.45, 0.6])
    base = rng.standard_normal((EL - SL, N, 2))
    gli = base.copy()
    cpro = ctypes.c_float(0)
    if form == "DT":
        typ, DW = zs[pick], dwv[pick]
        rc = lib.Potential_rec_DT_DW(a, b, gam, Nmult, Mmult, N, M, na, SL, EL, _p(xx), _p(yy), _p(DW),
                                     _p(ads), _p(occ), _p(typ), _p(gli), ctypes.byref(cpro))
        ref = O.muslib_rec_potential(a, b, gam, Nmult, Mmult, N, M, SL, EL, xx, yy, ads, occ, typ, DW=DW)
    else:
        typ = pick.astype(np.int32)
        curves = np.ascontiguousarray(O.create_pots(zs, dwv, 60, 0.02, vol=1 / (a * b * np.sin(gam))))
        rc = lib.Potential_rec_curve_DW(a, b, gam, Nmult, Mmult, N, M, na, SL, EL, _p(xx), _p(yy), _p(ads),
                                        _p(occ), _p(typ), _p(curves), 60, 0.02, _p(gli), ctypes.byref(cpro))
        ref = O.muslib_rec_potential(a, b, gam, Nmult, Mmult, N, M, SL, EL, xx, yy, ads, occ, typ,
                                     curves=curves, dds=0.02)
    assert rc == 0
    got = (gli[..., 0] - base[..., 0]) + 1j * (gli[..., 1] - base[..., 1])
    assert np.abs(ref).max() > 0.1
    np.testing.assert_allclose(got, ref, atol=1e-12 * np.abs(ref).max())
    rows = (SL == 0) + sum(1 for j in range(1, M) if j * Mmult < M // 2 and
                           (SL <= j * Mmult < EL or SL <= M - j * Mmult < EL))
    ref_p = np.float32(0)
    for _ in range(rows):
        ref_p = np.float32(np.float64(ref_p) + 200.0 / M)
    assert cpro.value == ref_p


# --------------------------------------- against the compiled reference's outputs
# tests/golden/muslib.npz: every export of the reference's Muslib compiled
# unchanged and run on seeded inputs (tests/golden/make_muslib_golden.py).

GAMS = (np.pi / 2, 1.8)


@pytest.mark.parametrize("name", _abi.MUSLIB_RS)
@pytest.mark.parametrize("gi", [0, 1])
def test_real_space_forms_vs_compiled_reference(golden, name, gi):
    import torch  # noqa: F401
    lib = _abi.load()
    G = golden("muslib.npz")
    kind, _, src, coord, _ = name.split("_")
    pre = f"rsin_{src}_{coord}_"
    a, b, E, atrad, N, M = G[pre + "scalars"]
    N, M = int(N), int(M)
    I = {k: np.ascontiguousarray(G[pre + k]) for k in ("xx", "yy", "ads", "occ", "dw", "typ", "curves")}
    gli = np.zeros((M, N, 2))
    if kind == "PG":
        gli[..., 0] = 1.0
    cpro = ctypes.c_float(0)
    head = (a, b, GAMS[gi], E, atrad) if kind == "PG" else (a, b, GAMS[gi], atrad)
    common = (N, M, len(I["xx"]), _p(I["xx"]), _p(I["yy"]))
    if src == "curve":
        tail = (_p(I["ads"]), _p(I["occ"]), _p(I["typ"]), _p(I["curves"]), I["curves"].shape[1], 0.01,
                _p(gli), ctypes.byref(cpro))
    elif coord == "DW":
        tail = (_p(I["dw"]), _p(I["ads"]), _p(I["occ"]), _p(I["typ"]), _p(gli), ctypes.byref(cpro))
    else:
        tail = (_p(I["ads"]), _p(I["occ"]), _p(I["typ"]), _p(gli), ctypes.byref(cpro))
    assert getattr(lib, name)(*head, *common, *tail) == 0
    ref = G[f"rs_{name}_{gi}_gli"]
    assert O.rel_l2(gli[..., 0] + 1j * gli[..., 1], ref[..., 0] + 1j * ref[..., 1]) < 1e-12
    assert cpro.value == float(G[f"rs_{name}_{gi}_cpro"])


@pytest.mark.parametrize("gi", [0, 1])
def test_propagator_vs_compiled_reference(golden, gi):
    import torch  # noqa: F401
    lib = _abi.load()
    G = golden("muslib.npz")
    a, b, gam, dz, E, tx, ty, N, M = G[f"prop_{gi}_args"]
    gli = np.zeros((int(M), int(N), 2))
    cpro = ctypes.c_float(-1)
    assert lib.CreatePropagator(a, b, gam, dz, E, tx, ty, int(N), int(M), _p(gli), ctypes.byref(cpro)) == 0
    np.testing.assert_allclose(gli, G[f"prop_{gi}_gli"], atol=1e-12)
    assert cpro.value == float(G[f"prop_{gi}_cpro"])


def test_one_atom_vs_compiled_reference(golden):
    import torch  # noqa: F401
    lib = _abi.load()
    G = golden("muslib.npz")
    cur = np.ascontiguousarray(G["oneatom_curve"])
    gli = np.zeros((40, 48, 2))
    gli[..., 0] = 1.0
    assert lib.PG_rs_curve_DW_cutpot_oneatom(8.0, 8.0, 1.9, 0.025, 1.0, 48, 40, 0.3, 0.7, 0.04, 0.9, _p(cur),
                                             500, 0.01, _p(gli)) == 0
    ref = G["oneatom_gli"]
    assert O.rel_l2(gli[..., 0] + 1j * gli[..., 1], ref[..., 0] + 1j * ref[..., 1]) < 1e-12


@pytest.mark.parametrize("ci", [0, 1, 2])
@pytest.mark.parametrize("form", ["DT", "curve"])
def test_reciprocal_space_vs_compiled_reference(golden, ci, form):
    import torch  # noqa: F401
    lib = _abi.load()
    G = golden("muslib.npz")
    gam, Nm, Mm, SL, EL = G[f"rec_{ci}_case"]
    Nm, Mm, SL, EL = int(Nm), int(Mm), int(SL), int(EL)
    xx, yy = np.ascontiguousarray(G["recin_xx"]), np.ascontiguousarray(G["recin_yy"])
    ads, occ = np.ascontiguousarray(G["recin_ads"]), np.ascontiguousarray(G["recin_occ"])
    zs, pick, dwv = G["recin_zs"], G["recin_pick"], G["recin_dwv"]
    na = len(xx)
    gli = np.zeros((EL - SL, 48, 2))
    cpro = ctypes.c_float(0)
    if form == "DT":
        typ = np.ascontiguousarray(zs[pick], np.int32)
        DW = np.ascontiguousarray(dwv[pick])
        rc = lib.Potential_rec_DT_DW(11.0, 12.0, gam, Nm, Mm, 48, 64, na, SL, EL, _p(xx), _p(yy), _p(DW),
                                     _p(ads), _p(occ), _p(typ), _p(gli), ctypes.byref(cpro))
    else:
        typ = np.ascontiguousarray(pick, np.int32)
        cur = np.ascontiguousarray(G[f"rec_{ci}_curves"])
        rc = lib.Potential_rec_curve_DW(11.0, 12.0, gam, Nm, Mm, 48, 64, na, SL, EL, _p(xx), _p(yy), _p(ads),
                                        _p(occ), _p(typ), _p(cur), 60, 0.02, _p(gli), ctypes.byref(cpro))
    assert rc == 0
    ref = G[f"rec_{ci}_{form}_gli"]
    np.testing.assert_allclose(gli, ref, atol=1e-12 * np.abs(ref).max())
    assert cpro.value == float(G[f"rec_{ci}_{form}_cpro"])


def test_curves_vs_compiled_reference(golden):
    lib = _abi.load()
    G = golden("muslib.npz")
    zq, sq, tab = G["scat_z"], G["scat_s"], G["scat_tab"]
    for i, z in enumerate(zq):
        for j, s_ in enumerate(sq):
            assert lib.scat_ampl_rs_DT_DW(int(z), float(s_), 0.4) == pytest.approx(tab[0, i, j], rel=1e-14, abs=0)
            assert lib.scat_ampl_rs2_DT_DW(int(z), float(s_), 0.4) == pytest.approx(tab[1, i, j], rel=1e-14, abs=0)
            assert lib.scat_ampl_rs2_DT_DW0(int(z), float(s_)) == pytest.approx(tab[2, i, j], rel=1e-14, abs=0)
    types, dws = np.ascontiguousarray(G["pots_types"]), np.ascontiguousarray(G["pots_dw"])
    for vol, key in ((0.0123, "pots_rec"), (None, "pots_rs")):
        sc = np.zeros((3, 80))
        if vol is None:
            lib.CreatePots_rs_DT_DW(3, 80, 0.015, _p(types), _p(dws), _p(sc))
        else:
            lib.CreatePots_rec_DT_DW(3, 80, 0.015, _p(types), _p(dws), vol, _p(sc))
        np.testing.assert_allclose(sc, G[key], rtol=1e-13, atol=0)
