"""The oracle's CTEM imaging (objective lens, defocus spread, partial coherence)
against the reference's own code: tests/golden/ctem_partial.npz holds images of
mulslice.cpp:539-676 driven by the reference's cfpix transforms and propagate()
and values of its chi() (slicelib.cpp:258-323), all compiled unchanged
(tests/golden/make_ctem_golden.py)."""
import numpy as np
import pytest

from oracle import msl_oracle as O


def lens_args(G, ci, lam):
    acmin, acmax, cs, df0, sigf, dfd, aobj, dfa2, dfa2p, dfa3, dfa3p = G["cases"][ci]
    return dict(acmin=acmin * 1e-3, acmax=acmax * 1e-3, cs=cs * 1e7, df=df0, df_spread=sigf, df_step=dfd,
                k_obj=float(np.float32(aobj * 1e-3) / np.float32(lam)),
                astig=(dfa2, np.radians(dfa2p), dfa3, np.radians(dfa3p)))


@pytest.mark.parametrize("ci", [0, 1, 2])
def test_partial_coherence_matches_reference(golden, ci):
    G = golden("ctem_partial.npz")
    S = golden("si_small.npz")
    ax, by, dz, kev = float(S["ax"]), float(S["by"]), float(S["dz"]), float(S["kev"])
    nx, ny = S["t"].shape[1:]
    lam = float(np.float32(O.wavelength(kev)))
    L = lens_args(G, ci, lam)
    props = [O.propagator_tables(nx, ny, ax, by, kev, dz, precision="f32")] * S["t"].shape[0]
    mask = O.band_mask(nx, ny, ax, by)
    img, nang = O.partial_coherence(S["t"].astype(np.complex128), props, S["seq"], mask, ax, by, kev, L["cs"],
                                    L["df"], L["k_obj"], L["acmin"], L["acmax"], L["df_spread"], L["df_step"],
                                    L["astig"])
    assert nang == int(G[f"pc_{ci}_nillum"])
    assert O.rel_l2(img, G[f"pc_{ci}_pix"]) < 2e-5


def test_chi_matches_reference_chi(golden):
    """chi() with Cs, defocus, C12a/b and C23a/b equals the library's (mulslice's)
    form with dfa2 = |C12|, 2 dfa2phi = atan2(-C12a, C12b), dfa3 = |C23|,
    3 dfa3phi = atan2(-C23a, C23b)."""
    G = golden("ctem_partial.npz")
    cs, df, c12a, c12b, c23a, c23b = G["chi_coef"].astype(np.float32).astype(np.float64)
    lam = O.wavelength(200.0)
    alx, aly = G["chi_alx"], G["chi_aly"]
    k2 = (alx * alx + aly * aly) / lam ** 2
    phi = np.arctan2(aly, alx)
    astig = (np.hypot(c12a, c12b), 0.5 * np.arctan2(-c12a, c12b), np.hypot(c23a, c23b),
             np.arctan2(-c23a, c23b) / 3.0)
    ours = O.chi(k2, phi, lam, cs, df, astig)
    ref = 2 * np.pi * G["chi_w"] / lam
    np.testing.assert_allclose(ours, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
