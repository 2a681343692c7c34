"""The batched FP64 oracle (oracle/fp64_gpu.py, torch complex128) against the
numpy oracle it restates, on the CPU at small sizes: potential, transmission,
probes, STEM detector sums and the frozen-phonon CTEM image."""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O

torch = pytest.importorskip("torch")
from oracle import fp64_gpu as G  # noqa: E402

CPU = torch.device("cpu")


def test_potential_matches_numpy_oracle(fparams):
    spec = S.srtio3(2, 2, 2, 3.905)
    ref = O.potential(spec.x, spec.y, spec.z, spec.Z, fparams, spec.ax, spec.by, spec.cz, 64, 64, 4, 3.0)
    got = G.potential(spec.x, spec.y, spec.z, spec.Z, fparams, spec.ax, spec.by, spec.cz, 64, 64, 4, 3.0,
                      CPU, chunk=7).numpy()
    assert np.abs(ref).max() > 10
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_stem_matches_numpy_oracle(fparams):
    spec = S.srtio3(2, 2, 2, 3.905)
    n, ns, kev = 64, 4, 200.0
    V = O.potential(spec.x, spec.y, spec.z, spec.Z, fparams, spec.ax, spec.by, spec.cz, n, n, ns, 3.0)
    T0 = O.transmission(V, kev, spec.ax, spec.by, np.complex128)
    T = G.transmission(torch.as_tensor(V), kev, spec.ax, spec.by)
    np.testing.assert_allclose(T.numpy(), T0, atol=1e-13)
    k_ap = float(S.mrad_to_k(25.0, kev))
    det = [(float(S.mrad_to_k(80, kev)), float(S.mrad_to_k(200, kev))),
           (float(S.mrad_to_k(11, kev)), float(S.mrad_to_k(22, kev)))]
    xy = S.raster(0.5 * 3.905, 1.5 * 3.905, 0.5 * 3.905, 1.5 * 3.905, 3, 2)
    P0 = O.probe(n, n, spec.ax, spec.by, kev, 0.0, k_ap, 0.0, 0.0, xy, np.complex128)
    P = G.probes(n, n, spec.ax, spec.by, kev, 0.0, k_ap, 0.0, 0.0, xy, CPU)
    np.testing.assert_allclose(P.numpy(), P0, atol=1e-14)
    props = [O.propagator_tables(n, n, spec.ax, spec.by, kev, spec.cz / ns, precision="f64")] * ns
    ref = O.stem(T0, props, np.arange(ns), O.band_mask(n, n, spec.ax, spec.by), P0,
                 O.detector_masks(n, n, spec.ax, spec.by, det), [1, 3])
    prop = G.propagator(n, n, spec.ax, spec.by, kev, spec.cz / ns, CPU)
    got = G.stem_scan(T, prop, np.arange(ns), n, n, spec.ax, spec.by, kev, k_ap, xy, det, [1, 3], batch=4)
    np.testing.assert_allclose(got, ref, rtol=1e-11)


def test_frozen_phonon_matches_numpy_oracle(fparams):
    spec = S.fcc_au(2, 2, 2)
    n, ns, kev, cs, df, k_obj = 64, 4, 300.0, 1.2e7, -600.0, 2.0
    img, exi = G.frozen_phonon(spec, fparams, n, n, ns, 3.0, kev, cs, df, k_obj, 2, 0.085, 3, CPU)
    ri, re_ = np.zeros((n, n)), np.zeros((n, n))
    mask = O.band_mask(n, n, spec.ax, spec.by)
    props = [O.propagator_tables(n, n, spec.ax, spec.by, kev, spec.cz / ns, precision="f64")] * ns
    for c in range(2):
        d = O.phonon_displacements(3, c, spec.natom, 0.085)
        V = O.potential(spec.x + d[:, 0], spec.y + d[:, 1], spec.z + d[:, 2], spec.Z, fparams, spec.ax,
                        spec.by, spec.cz, n, n, ns, 3.0)
        T = O.transmission(V, kev, spec.ax, spec.by, np.complex128)
        w, _ = O.multislice(np.ones((n, n), np.complex128), T, props, np.arange(ns), mask)
        ri += O.ctem_image(w, spec.ax, spec.by, kev, cs, df, k_obj) / 2
        re_ += np.abs(w) ** 2 / 2
    np.testing.assert_allclose(exi, re_, rtol=1e-11)
    np.testing.assert_allclose(img, ri, rtol=1e-11)
