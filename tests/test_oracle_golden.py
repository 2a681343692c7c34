"""Pin the numpy oracle against golden vectors made by the reference's own code.

The golden vectors (tests/golden/make_golden.py) come from Kirkland's cfpix.cpp
and slicelib.cpp compiled unchanged over the vendored FFTW 2.1.5 (float).
"""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O


def test_vzatom_and_constants(golden, fparams):
    g = golden("vzatom.npz")
    v = np.array([[O.vzatom(int(z), r, fparams) for r in g["r"]] for z in g["Z"]])
    np.testing.assert_allclose(v, g["vz"], rtol=1e-13)
    np.testing.assert_allclose(O.wavelength(g["kev"]), g["wavelength"], rtol=1e-15)
    np.testing.assert_allclose(O.sigma(g["kev"]), g["sigma"], rtol=1e-15)


def test_potential_small(golden, fparams):
    G = golden("si_small.npz")
    spec = S.si_diamond(2, 2, 2, 5.431)
    V = O.potential(spec.x, spec.y, spec.z, spec.Z, fparams, spec.ax, spec.by, spec.cz, 64, 64, 8, 3.0)
    np.testing.assert_allclose(V, G["v"], rtol=1e-12, atol=1e-9)


def test_transmission_and_ctem_small(golden):
    G = golden("si_small.npz")
    ax, by = float(G["ax"]), float(G["by"])
    T = O.transmission(G["v"], 200.0, ax, by, np.complex64)
    assert O.rel_l2(T, G["t"]) < 1e-6
    mask = O.band_mask(64, 64, ax, by)
    props = [O.propagator_tables(64, 64, ax, by, 200.0, float(G["dz"]), precision="f32")] * 8
    w, _ = O.multislice(np.ones((64, 64), np.complex64), T, props, G["seq"], mask)
    assert O.rel_l2(w, G["wave"]) < 1e-5


def test_ctem_config1_fp64_oracle_vs_reference(golden, fparams):
    """The FP64 oracle and the reference's FP32 mulslice agree on the Si 256^2 exit wave."""
    C = golden("si_config1.npz")
    cfg = S.config_si_ctem()
    spec = cfg["spec"]
    V = O.potential(spec.x, spec.y, spec.z, spec.Z, fparams, spec.ax, spec.by, spec.cz,
                    256, 256, 80, cfg["radius"])
    np.testing.assert_allclose([V.sum(), (V ** 2).sum()], C["v_checksum"], rtol=1e-12)
    mask = O.band_mask(256, 256, spec.ax, spec.by)
    T = O.transmission(V, 200.0, spec.ax, spec.by, np.complex128)
    props = [O.propagator_tables(256, 256, spec.ax, spec.by, 200.0, spec.cz / 80, precision="f64")]
    w, _ = O.multislice(np.ones((256, 256), np.complex128), T, props * 80, np.arange(80), mask)
    assert O.rel_l2(w, C["wave"]) < 2e-5


def test_stem_small(golden):
    G = golden("stem_small.npz")
    ax, by, kev, dz = float(G["ax"]), float(G["by"]), float(G["kev"]), float(G["dz"])
    T = O.transmission(G["v"].astype(np.float64), kev, ax, by, np.complex64)
    props = [O.propagator_tables(128, 128, ax, by, kev, dz, precision="f32")] * 20
    mask = O.band_mask(128, 128, ax, by)
    P = O.probe(128, 128, ax, by, kev, 0.0, float(G["k_ap"]), 0.0, 0.0, G["xy"], np.complex64)
    dm = O.detector_masks(128, 128, ax, by, G["det_k"])
    r = O.stem(T, props, np.arange(20), mask, P, dm, list(G["cps"]))
    assert O.rel_l2(r, G["det"]) < 1e-5


def test_oracle_fft_convention():
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((8, 16)) + 1j * rng.standard_normal((8, 16))).astype(np.complex128)
    n = np.arange(8)[:, None, None, None] * np.arange(8)[None, None, :, None] / 8.0
    m = np.arange(16)[None, :, None, None] * np.arange(16)[None, None, None, :] / 16.0
    # direct sum with exp(+2 pi i ...), unscaled
    ref = np.einsum("xy,xyab->ab", x, np.exp(2j * np.pi * (n + m)))
    np.testing.assert_allclose(O.kfft(x), ref, atol=1e-10)
    np.testing.assert_allclose(O.kifft(O.kfft(x)), x, atol=1e-12)


@pytest.mark.parametrize("n,a", [(64, 10.0), (100, 7.0), (255, 3.3)])
def test_freqn_matches_reference_rule(n, a):
    k, k2 = O.freqn(n, a)
    imid = int(n / 2.0 + 0.5)
    for i in (0, 1, imid, imid + 1, n - 1):
        ref = np.float32(i if i <= imid else i - n) / np.float32(a)
        assert k[i] == ref and k2[i] == np.float32(ref * ref)
