"""Known-answer checks of the GPU path that need no reference output: the
analytic Fresnel spreading of a Gaussian, unitarity of the vacuum slice step,
the mirror symmetry of STEM on a centro-symmetric crystal, and a single atom's
projected potential against the parameterised formula itself."""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def test_fresnel_propagation_of_a_gaussian(ctx):
    """exp(-x^2/2s^2) after a vacuum thickness z is (s/sqrt(q)) exp(-x^2/2q) per axis,
    q = s^2 + i lambda z / 2 pi (Kirkland's propagator sign)."""
    n, a, kev, s = 256, 25.6, 200.0, 1.5
    x = (np.arange(n) - n // 2) * a / n
    g = np.exp(-x ** 2 / (2 * s ** 2))
    psi = (g[:, None] * g[None, :]).astype(np.complex64)[None]
    nsl, dz = 20, 10.0
    w = ctx.multislice(np.ones((1, n, n), np.complex64), dz, [0] * nsl, a, a, kev, psi=psi.copy())[0]
    q = s ** 2 + 1j * O.wavelength(kev) * nsl * dz / (2 * np.pi)
    g1 = (s / np.sqrt(q)) * np.exp(-x ** 2 / (2 * q))
    assert O.rel_l2(w, g1[:, None] * g1[None, :]) < 2e-5


def test_vacuum_slice_step_is_unitary(ctx):
    """Inside the band limit every propagation step keeps the norm of the wave."""
    n, a, kev = 128, 16.0, 300.0
    rng = np.random.default_rng(3)
    w = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    spec = O.kfft(w) * O.band_mask(n, n, a, a)                 # band-limited start
    psi = O.kifft(spec).astype(np.complex64)[None]
    norm0 = np.linalg.norm(psi.astype(np.complex128))
    out = ctx.multislice(np.ones((1, n, n), np.complex64), 2.5, [0] * 50, a, a, kev, psi=psi.copy())
    assert abs(np.linalg.norm(out.astype(np.complex128)) / norm0 - 1.0) < 1e-5


def test_stem_mirror_symmetry_on_centrosymmetric_crystal(ctx):
    """SrTiO3 [001] is mirror-symmetric about a Sr column and the atoms sit on grid
    points, so probes at x0 +- d on either side of a column give equal signals."""
    spec = S.srtio3(4, 4, 6)
    nx = 256
    v = ctx.potential(spec, nx, nx, 12, 1.9)
    t = ctx.transmission(v, spec.ax, spec.by, 200.0)
    px = spec.ax / nx
    x0, y0 = 2 * 3.905, 2 * 3.905                               # a Sr column
    xy = np.array([[x0 + 5 * px, y0 + 3 * px], [x0 - 5 * px, y0 + 3 * px],
                   [x0 + 5 * px, y0 - 3 * px], [x0 + 3 * px, y0 + 5 * px]])
    k_ap = float(S.mrad_to_k(20.0, 200.0))
    det = [(float(S.mrad_to_k(60.0, 200.0)), float(S.mrad_to_k(150.0, 200.0))), (0.0, k_ap)]
    d = ctx.stem_scan(t, spec.cz / 12, np.arange(12), spec.ax, spec.by, 200.0, k_ap, xy, det)[:, 0, :]
    assert d[0, 0] > 0
    for k in range(1, 4):                                       # mirrors in x, y and the diagonal
        np.testing.assert_allclose(d[k], d[0], rtol=2e-5)


def test_single_atom_potential_matches_formula(ctx, fparams):
    """One gold atom: every pixel within the cutoff carries vzatom(79, r), none beyond."""
    a, n, radius = 20.0, 128, 4.0
    x0, y0 = 10.03, 9.98
    spec = S.Specimen(np.array([x0]), np.array([y0]), np.array([1.0]), np.array([79], np.int32), a, a, 2.0)
    v = ctx.potential(spec, n, n, 1, radius)[0].astype(np.float64)
    g = np.arange(n) * a / n
    r = np.sqrt((g[:, None] - x0) ** 2 + (g[None, :] - y0) ** 2)
    inside = r < radius
    ref = O.vzatom(79, r[inside], fparams)
    np.testing.assert_allclose(v[inside], ref, rtol=2e-5, atol=1e-6 * ref.max())
    assert np.all(v[~inside] == 0)
