"""The slice loop's passes on every kernel family: two-stage columns at 256,
512 and 1024 (swizzled TMA tiles, independent thread groups per CTA; at 1024 a
column is shared by a warp pair), mixed-radix 384 / 768 rows and columns, the
2048 warp-pair rows; non-square grids, batches that leave groups without
tiles, several detectors and checkpoints, against the FP64 oracle."""
import numpy as np
import pytest

from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def _layers(rng, nt, nx, ny, ax, by, kev):
    v = np.zeros((nt, nx, ny))
    for l in range(nt):
        ix = rng.integers(0, nx, 24)
        iy = rng.integers(0, ny, 24)
        v[l, ix, iy] = rng.uniform(50, 400, 24)
    return O.transmission(v, kev, ax, by, np.complex64)


@pytest.mark.parametrize("nx,ny,batch", [(256, 64, 1), (256, 384, 3), (256, 256, 7),
                                         (512, 64, 1), (512, 384, 3), (512, 1024, 2), (512, 512, 5),
                                         (1024, 64, 1), (1024, 256, 3), (1024, 1024, 2),
                                         (384, 768, 2), (768, 384, 3), (768, 2048, 1), (2048, 768, 1)])
def test_ctem_two_stage_columns_match_oracle(ctx, nx, ny, batch):
    rng = np.random.default_rng(nx + ny + batch)
    ax, by, kev = 30.0, 30.0 * ny / nx, 200.0
    t = _layers(rng, 3, nx, ny, ax, by, kev)
    dz = np.array([1.2, 1.9, 1.5])
    seq = [0, 1, 2, 1, 0, 2, 2]
    psi = (rng.standard_normal((batch, nx, ny)) + 1j * rng.standard_normal((batch, nx, ny))).astype(np.complex64)
    got = ctx.multislice(t, dz, seq, ax, by, kev, psi=psi.copy())
    props = [O.propagator_tables(nx, ny, ax, by, kev, d, precision="f64") for d in dz]
    ref, _ = O.multislice(psi.astype(np.complex128), t.astype(np.complex128), props, seq,
                          O.band_mask(nx, ny, ax, by))
    assert O.rel_l2(got, ref) < 2e-5


@pytest.mark.parametrize("nx,ny", [(256, 256), (512, 384), (1024, 256), (384, 768), (768, 384), (2048, 64)])
def test_stem_two_stage_columns_detectors_and_checkpoints(ctx, nx, ny):
    rng = np.random.default_rng(11)
    ax, kev = 31.0 * nx / 512, 200.0  # 0.06 A pixels: every detector inside the band limit
    by = ax * ny / nx
    t = _layers(rng, 2, nx, ny, ax, by, kev)
    seq = [0, 1, 0, 1, 1, 0]
    k_ap = 1.5
    xy = rng.uniform(0, [ax, by], (5, 2))
    det = [(0.0, 0.5), (0.5, 1.2), (1.2, 2.0), (2.0, 3.0), (3.0, 4.5)]
    cps = [1, 3, 5]
    d = ctx.stem_scan(t, 1.6, seq, ax, by, kev, k_ap, xy, det, checkpoints=cps)
    props = [O.propagator_tables(nx, ny, ax, by, kev, 1.6, precision="f64")] * 2
    probes = O.probe(nx, ny, ax, by, kev, 0.0, k_ap, 0.0, 0.0, xy, np.complex128)
    ref = O.stem(t.astype(np.complex128), props, seq, O.band_mask(nx, ny, ax, by), probes,
                 O.detector_masks(nx, ny, ax, by, det), cps)
    assert d.shape == ref.shape == (5, 3, 5)
    assert O.rel_l2(d, ref) < 2e-5
    for k in range(len(det)):
        assert O.rel_l2(d[..., k], ref[..., k]) < 1e-3  # the STEM image bar
