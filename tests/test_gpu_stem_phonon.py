"""GPU parity of frozen-phonon STEM: the thermal-vibration loop the reference
wraps around every probe (MSProjectUseOnce.cs:235-273, jitter
MSUseOnceCalculator.cs:179-199), whose detector sums are added over the
configurations (MSProject.cs:836-837)."""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu

KEV = 200.0
A = 3.905


def _setup(n=128):
    spec = S.srtio3(2, 2, 4, A)
    k_ap = float(S.mrad_to_k(25.0, KEV))
    det = [(float(S.mrad_to_k(80, KEV)), float(S.mrad_to_k(200, KEV))),
           (float(S.mrad_to_k(11, KEV)), float(S.mrad_to_k(22, KEV)))]
    xy = S.raster(0.5 * A, 1.5 * A, 0.5 * A, 1.5 * A, 3, 2)
    return spec, k_ap, det, xy


def _oracle(spec, fp, n, nslice, k_ap, xy, det, nconfig, sigma, seed, checkpoints):
    mask = O.band_mask(n, n, spec.ax, spec.by)
    props = [O.propagator_tables(n, n, spec.ax, spec.by, KEV, spec.cz / nslice, precision="f64")] * nslice
    P = O.probe(n, n, spec.ax, spec.by, KEV, 0.0, k_ap, 0.0, 0.0, xy, np.complex128)
    dm = O.detector_masks(n, n, spec.ax, spec.by, det)
    tot = 0.0
    for c in range(nconfig):
        d = O.phonon_displacements(seed, c, spec.natom, sigma)
        V = O.potential(spec.x + d[:, 0], spec.y + d[:, 1], spec.z + d[:, 2], spec.Z, fp, spec.ax,
                        spec.by, spec.cz, n, n, nslice, 3.0)
        T = O.transmission(V, KEV, spec.ax, spec.by, np.complex128)
        tot = tot + O.stem(T, props, np.arange(nslice), mask, P, dm, checkpoints)
    return tot


def test_stem_phonon_vs_oracle(ctx, fparams):
    spec, k_ap, det, xy = _setup()
    got = ctx.stem_scan_phonon(spec, 128, 128, 8, 3.0, KEV, k_ap, xy, det, nconfig=3, sigma=0.085,
                               seed=5, checkpoints=[3, 7])
    ref = _oracle(spec, fparams, 128, 8, k_ap, xy, det, 3, 0.085, 5, [3, 7])
    assert got.shape == (len(xy), 2, 2)
    for k in range(2):
        for d in range(2):
            assert O.rel_l2(got[:, k, d], ref[:, k, d]) < 1e-4


def test_stem_phonon_one_config_zero_sigma_equals_static_scan(ctx):
    """sigma = 0 and one configuration is the plain scan of the same slices."""
    spec, k_ap, det, xy = _setup()
    got = ctx.stem_scan_phonon(spec, 128, 128, 8, 3.0, KEV, k_ap, xy, det, nconfig=1, sigma=0.0, seed=1)
    v = ctx.potential(spec, 128, 128, 8, 3.0)
    t = ctx.transmission(v, spec.ax, spec.by, KEV)
    ref = ctx.stem_scan(t, spec.cz / 8, np.arange(8), spec.ax, spec.by, KEV, k_ap, xy, det)
    assert np.array_equal(got, ref)


def test_stem_phonon_sums_do_not_depend_on_batching():
    """Probes x configurations share one slice loop; neither the probe batch nor
    a memory cap that splits the configurations into batches changes any sum."""
    from multislice_gb300 import Context
    spec, k_ap, det, xy = _setup()
    args = (spec, 128, 128, 8, 3.0, KEV, k_ap, xy, det)
    kw = dict(nconfig=4, sigma=0.085, seed=9, checkpoints=[2, 7])
    with Context(0) as c:
        l0 = c.launches
        full = c.stem_scan_phonon(*args, **kw)
        batched = c.launches - l0
    with Context(0) as c:
        c.set_probe_batch(2)
        pb = c.stem_scan_phonon(*args, **kw)
    with Context(0) as c:
        # one configuration's transmissions: 1 MiB; a 4 MiB cap leaves 2 MiB for
        # them, so two configurations per batch instead of four
        c.set_memory_limit(4 << 20)
        l0 = c.launches
        one = c.stem_scan_phonon(*args, **kw)
        single = c.launches - l0
        assert c.memory_in_use() <= 4 << 20
    assert single > batched
    assert np.array_equal(full, pb)
    assert np.array_equal(full, one)


def test_stem_phonon_rejects_bad_arguments(ctx):
    from multislice_gb300 import MslError
    spec, k_ap, det, xy = _setup()
    with pytest.raises(MslError):
        ctx.stem_scan_phonon(spec, 128, 128, 8, 3.0, KEV, k_ap, xy, det, nconfig=0, sigma=0.1, seed=1)
    with pytest.raises(MslError):
        ctx.stem_scan_phonon(spec, 128, 128, 8, 3.0, KEV, k_ap, xy, det, nconfig=2, sigma=-1.0, seed=1)
    with pytest.raises(MslError):
        ctx.stem_scan_phonon(spec, 128, 128, 8, 3.0, KEV, k_ap, xy, det, nconfig=2, sigma=0.1, seed=1,
                             checkpoints=[9])
