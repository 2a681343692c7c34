"""The vectorised Muslib restatement (nine clipped rectangles per atom) against
a literal per-pixel loop over the same index ranges, PG_RS.cpp:57-119 (clipped)
and :304-446 (periodic), on a small cell."""
import math

import numpy as np
import pytest

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
