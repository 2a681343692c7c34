"""The vectorised Muslib restatement (nine clipped rectangles per atom) against
a literal per-pixel loop over the same index ranges, PG_RS.cpp:57-119 (clipped)
and :304-446 (periodic), on a small cell."""
import ctypes
import math
import os

import numpy as np
import pytest

from multislice_gb300 import _abi
from oracle import msl_oracle as O


def _loop_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic):
    sg, cg = math.sin(gam), math.cos(gam)
    drax, dray = atrad * sg / a, atrad * sg / b
    dxa, dyb = a / N, b / M
    npts = curves.shape[1]
    A = np.zeros((M, N))
    B = np.zeros((M, N))
    for k in range(len(xx)):
        ibb, iee = int((xx[k] - drax) * N), int((xx[k] + drax) * N)
        jbb, jee = int((yy[k] - dray) * M), int((yy[k] + dray) * M)
        if periodic:
            # the wrapped strip past the upper edge keeps one more pixel (:352, :365)
            irange = range(ibb, iee + (1 if iee >= N else 0))
            jrange = range(jbb, jee + (1 if jee >= M else 0))
        else:
            irange = range(max(ibb, 0), min(iee, N))
            jrange = range(max(jbb, 0), min(jee, M))
        for j in jrange:
            y = j * dyb - yy[k] * b
            for i in irange:
                x = i * dxa - xx[k] * a
                ar2 = math.sqrt(x * (x + 2 * y * cg) + y * y) / dds
                jj = math.floor(ar2)
                if jj >= npts - 1:
                    continue
                c = curves[typ[k]]
                res = c[jj] + (c[jj + 1] - c[jj]) * (ar2 - jj)
                A[j % M, i % N] += res * occ[k]
                B[j % M, i % N] += res * occ[k] * ads[k]
    return A, B


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("gam", [math.pi / 2, 1.8])
def test_curve_sums_match_literal_loop(periodic, gam):
    rng = np.random.default_rng(4)
    a, b, atrad, N, M, na, npts, dds = 6.0, 7.0, 1.5, 24, 28, 9, 200, 0.01
    xx = rng.random(na)
    yy = rng.random(na)
    xx[:3] = [0.02, 0.97, 0.5]
    yy[:3] = [0.03, 0.5, 0.99]
    ads = rng.random(na) * 0.05
    occ = 0.5 + 0.5 * rng.random(na)
    typ = rng.integers(0, 2, na)
    r = np.arange(npts) * dds
    curves = np.stack([np.exp(-r / 0.3), 2.0 * np.exp(-r / 0.5)])
    got = O.muslib_curve_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic)
    ref = _loop_sums(a, b, gam, atrad, N, M, xx, yy, ads, occ, typ, curves, dds, periodic)
    np.testing.assert_allclose(got[0], ref[0], atol=1e-12)
    np.testing.assert_allclose(got[1], ref[1], atol=1e-12)
    assert ref[0].max() > 0.5


def test_periodic_grating_adds_only_the_wrapped_parts():
    rng = np.random.default_rng(3)
    a, b, atrad, N, M, na, npts, dds = 10.0, 11.0, 2.0, 96, 128, 40, 400, 0.01
    xx, yy = rng.random(na), rng.random(na)
    xx[:2], yy[:2] = [0.01, 0.99], [0.01, 0.98]
    ads, occ = rng.random(na) * 0.05, 0.5 + 0.5 * rng.random(na)
    typ = rng.integers(0, 3, na)
    r = np.arange(npts) * dds
    curves = np.stack([z * np.exp(-r / 0.4) for z in (1.0, 2.0, 3.5)])
    args = (a, b, math.pi / 2, atrad, N, M, xx, yy, ads, occ, typ, curves, dds)
    per = O.muslib_curve_sums(*args, True)[0]
    cut = O.muslib_curve_sums(*args, False)[0]
    assert np.all(per >= cut - 1e-12) and (per - cut).max() > 0.1


def _lib():
    if not os.path.exists(_abi.LIB_PATH):
        from multislice_gb300 import build
        build.build()
    return _abi.load()


def test_doyle_turner_table_shape():
    tab = O.doyle_turner()
    assert tab.shape == (93, 8) and np.all(tab[0] == 0)
    assert tab[14, 0] == 2.1293 and tab[79, 7] == 0.3067   # Si a1, Au b4


def test_host_scattering_functions_match_oracle():
    """Curves.cpp host exports (no GPU needed) against the restatement."""
    lib = _lib()
    for z in (1, 6, 14, 38, 79, 92):
        for s, dw in ((0.0, 0.0), (0.05, 0.3), (0.7, 1.1)):
            assert lib.scat_ampl_rs2_DT_DW(z, s, dw) == pytest.approx(float(O.dt_rs2(z, s, dw)), rel=1e-14)
            assert lib.scat_ampl_rs_DT_DW(z, s, dw) == pytest.approx(float(O.dt_rs(z, s, dw)), rel=1e-14)
        assert lib.scat_ampl_rs2_DT_DW0(z, 0.2) == pytest.approx(float(O.dt_rs2(z, 0.2, 0.0)), rel=1e-14)
    types = np.array([6, 14, 79], np.int32)
    dw = np.array([0.3, 0.5, 0.0])
    npts, dds = 300, 0.01
    sc = np.zeros((3, npts))
    lib.CreatePots_rs_DT_DW(3, npts, dds, types.ctypes.data, dw.ctypes.data, sc.ctypes.data)
    np.testing.assert_allclose(sc, O.create_pots(types, dw, npts, dds), rtol=1e-13)
    lib.CreatePots_rec_DT_DW(3, npts, dds, types.ctypes.data, dw.ctypes.data, 0.02, sc.ctypes.data)
    np.testing.assert_allclose(sc, O.create_pots(types, dw, npts, dds, vol=0.02), rtol=1e-13)


def test_rec_potential_single_atom_closed_form():
    """One atom: the coefficient of reflection (h, k) is f(|g|/2) exp(-DW |g|^2/4)
    occ (1 + i ads) / area * exp(-2 pi i (h x + k y)), |g| on the reciprocal lattice
    of the oblique cell (angle pi - gam between a* and b*)."""
    a, b, gam, N, M = 7.0, 9.0, 1.7, 16, 20
    xx, yy = np.array([0.23]), np.array([0.61])
    ads, occ, typ, DW = np.array([0.07]), np.array([0.8]), np.array([29]), np.array([0.4])
    got = O.muslib_rec_potential(a, b, gam, 1, 1, N, M, 0, M, xx, yy, ads, occ, typ, DW=DW)
    A_, B_ = 1 / (a * math.sin(gam)), 1 / (b * math.sin(gam))
    vol = 1 / (a * b * math.sin(gam))
    for h in range(-N // 2 + 1, N // 2):
        for k in range(-M // 2 + 1, M // 2):
            g2 = (h * A_) ** 2 + (k * B_) ** 2 - 2 * h * k * A_ * B_ * math.cos(gam)
            s = math.sqrt(g2) / 2
            ref = (O.dt_rec(29, s) * math.exp(-DW[0] * s * s) * vol * occ[0] * (1 + 1j * ads[0]) *
                   np.exp(-2j * math.pi * (h * xx[0] + k * yy[0])))
            assert abs(got[k % M, h % N] - ref) < 1e-12 * max(1.0, abs(ref)), (h, k)
    assert np.all(got[M // 2] == 0) and np.all(got[:, N // 2] == 0)   # Nyquist lines are never written


def test_rec_potential_curve_band_and_symmetry():
    """Without absorption the coefficients are Hermitian, and a row band [SL, EL)
    equals the same rows of the full grid."""
    rng = np.random.default_rng(5)
    a, b, gam, N, M, na = 8.0, 8.0, math.pi / 2, 24, 24, 6
    xx, yy = rng.random(na), rng.random(na)
    occ, typ = 0.5 + 0.5 * rng.random(na), rng.integers(0, 2, na)
    curves = O.create_pots([8, 38], [0.2, 0.4], 500, 0.005, vol=1 / (a * b))
    full = O.muslib_rec_potential(a, b, gam, 1, 1, N, M, 0, M, xx, yy, np.zeros(na), occ, typ,
                                  curves=curves, dds=0.005)
    for jj in range(1, M // 2):
        for ii in range(1, N // 2):
            assert abs(full[M - jj, N - ii] - np.conj(full[jj, ii])) < 1e-12
    band = O.muslib_rec_potential(a, b, gam, 1, 1, N, M, 5, 19, xx, yy, np.zeros(na), occ, typ,
                                  curves=curves, dds=0.005)
    np.testing.assert_allclose(band, full[5:19], atol=1e-13)
    dt = O.muslib_rec_potential(a, b, gam, 1, 1, N, M, 0, M, xx, yy, np.zeros(na), occ,
                                np.array([8, 38])[typ], DW=np.array([0.2, 0.4])[typ])
    assert O.rel_l2(full, dt) < 1e-4      # the tabulated curve approximates the DT form


# ------------------------------------------------- against the compiled reference
# tests/golden/muslib.npz holds the outputs of the reference's own Muslib sources
# compiled unchanged (tests/golden/make_muslib_golden.py); the restatement must
# reproduce them to rounding.

RS_NAMES = [f"{k}_rs_{s}_{c}_{w}" for k in ("PG", "Potential") for s in ("curve", "DT") for c in ("DW", "TV")
            for w in ("cutpot", "periodic")]
GAMS = (np.pi / 2, 1.8)


def muslib_case(G, name):
    """Inputs of one real-space form from the fixture."""
    _, _, src, coord, _ = name.split("_")
    pre = f"rsin_{src}_{coord}_"
    a, b, E, atrad, N, M = G[pre + "scalars"]
    inp = {k: G[pre + k] for k in ("xx", "yy", "ads", "occ", "dw", "typ", "curves")}
    return float(a), float(b), float(E), float(atrad), int(N), int(M), inp


def restated_rs(name, gam, G):
    kind, _, src, coord, wrap = name.split("_")
    a, b, E, atrad, N, M, I = muslib_case(G, name)
    A, B = O.muslib_rs_sums(a, b, gam, atrad, N, M, I["xx"], I["yy"], I["ads"], I["occ"], I["typ"],
                            curves=I["curves"] if src == "curve" else None, dds=0.01, dw=I["dw"],
                            source="curve" if src == "curve" else f"DT_{coord}", angstrom=coord == "TV",
                            periodic=wrap == "periodic")
    if kind == "PG":
        return O.muslib_pg(A, B, E)
    return A + 1j * B


@pytest.mark.parametrize("name", RS_NAMES)
@pytest.mark.parametrize("gi", [0, 1])
def test_restatement_matches_compiled_muslib_real_space(golden, name, gi):
    G = golden("muslib.npz")
    ref = G[f"rs_{name}_{gi}_gli"]
    got = restated_rs(name, GAMS[gi], G)
    r = ref[..., 0] + 1j * ref[..., 1]
    assert np.abs(r).max() > 0.5
    assert O.rel_l2(got, r) < 1e-12


@pytest.mark.parametrize("gi", [0, 1])
def test_restatement_matches_compiled_muslib_propagator(golden, gi):
    G = golden("muslib.npz")
    a, b, gam, dz, E, tx, ty, N, M = G[f"prop_{gi}_args"]
    ref = G[f"prop_{gi}_gli"]
    got = O.muslib_propagator(a, b, gam, dz, E, tx, ty, int(N), int(M))
    np.testing.assert_allclose(got, ref[..., 0] + 1j * ref[..., 1], atol=1e-12)
    assert float(G[f"prop_{gi}_cpro"]) == 100.0


@pytest.mark.parametrize("ci", [0, 1, 2])
@pytest.mark.parametrize("form", ["DT", "curve"])
def test_restatement_matches_compiled_muslib_reciprocal(golden, ci, form):
    G = golden("muslib.npz")
    gam, Nm, Mm, SL, EL = G[f"rec_{ci}_case"]
    Nm, Mm, SL, EL = int(Nm), int(Mm), int(SL), int(EL)
    xx, yy, ads, occ = G["recin_xx"], G["recin_yy"], G["recin_ads"], G["recin_occ"]
    zs, pick, dwv = G["recin_zs"], G["recin_pick"], G["recin_dwv"]
    if form == "DT":
        got = O.muslib_rec_potential(11.0, 12.0, gam, Nm, Mm, 48, 64, SL, EL, xx, yy, ads, occ, zs[pick],
                                     DW=dwv[pick])
    else:
        cur = G[f"rec_{ci}_curves"]
        np.testing.assert_allclose(O.create_pots(zs, dwv, 60, 0.02, vol=1 / (11.0 * 12.0 * np.sin(gam))), cur,
                                   rtol=1e-13, atol=0)
        got = O.muslib_rec_potential(11.0, 12.0, gam, Nm, Mm, 48, 64, SL, EL, xx, yy, ads, occ,
                                     pick.astype(np.int32), curves=cur, dds=0.02)
    ref = G[f"rec_{ci}_{form}_gli"]
    r = ref[..., 0] + 1j * ref[..., 1]
    assert np.abs(r).max() > 0.1
    np.testing.assert_allclose(got, r, atol=1e-12 * np.abs(r).max())


def test_restatement_matches_compiled_muslib_curves(golden):
    G = golden("muslib.npz")
    zq, sq, tab = G["scat_z"], G["scat_s"], G["scat_tab"]
    for i, z in enumerate(zq):
        np.testing.assert_allclose(O.dt_rs(int(z), sq, 0.4), tab[0, i], rtol=1e-14, atol=0)
        np.testing.assert_allclose(O.dt_rs2(int(z), sq, 0.4), tab[1, i], rtol=1e-14, atol=0)
        np.testing.assert_allclose(O.dt_rs2(int(z), sq, 0.0), tab[2, i], rtol=1e-14, atol=0)
    types, dws = G["pots_types"], G["pots_dw"]
    np.testing.assert_allclose(O.create_pots(types, dws, 80, 0.015, vol=0.0123), G["pots_rec"], rtol=1e-13)
    np.testing.assert_allclose(O.create_pots(types, dws, 80, 0.015), G["pots_rs"], rtol=1e-13)


def test_restatement_matches_compiled_muslib_one_atom(golden):
    G = golden("muslib.npz")
    cur = G["oneatom_curve"]
    A, B = O.muslib_rs_sums(8.0, 8.0, 1.9, 1.0, 48, 40, np.array([0.3]), np.array([0.7]), np.array([0.04]),
                            np.array([0.9]), np.array([0]), curves=cur[None], dds=0.01, periodic=False,
                            whole=True)
    ref = G["oneatom_gli"]
    assert O.rel_l2(O.muslib_pg(A, B, 0, K=0.025), ref[..., 0] + 1j * ref[..., 1]) < 1e-12
