"""The on-chip STEM slice loop (msl_stem_scan_resident: one 8-CTA cluster per
probe, the 256^2 wave in distributed shared memory across all slices) against
the streaming scan and the FP64 oracle."""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu

KEV = 200.0
A = 3.905


def _case(ctx, ncells_z=20, nslice=40):
    spec = S.srtio3(4, 4, ncells_z, A)
    v = ctx.potential(spec, 256, 256, nslice, 3.0)
    t = ctx.transmission(v, spec.ax, spec.by, KEV)
    k_ap = float(S.mrad_to_k(25.0, KEV))
    det = [(float(S.mrad_to_k(80, KEV)), float(S.mrad_to_k(200, KEV))),
           (float(S.mrad_to_k(11, KEV)), float(S.mrad_to_k(22, KEV)))]
    return spec, t, k_ap, det


def test_resident_matches_streaming_scan_and_fp64(ctx):
    spec, t, k_ap, det = _case(ctx)
    xy = S.raster(1.5 * A, 2.5 * A, 1.5 * A, 2.5 * A, 5, 5)   # 25 probes: not a multiple of the clusters
    seq = np.arange(40)
    cps = [9, 24, 39]
    got = ctx.stem_scan(t, spec.cz / 40, seq, spec.ax, spec.by, KEV, k_ap, xy, det, checkpoints=cps, resident=True)
    ref = ctx.stem_scan(t, spec.cz / 40, seq, spec.ax, spec.by, KEV, k_ap, xy, det, checkpoints=cps)
    assert got.shape == ref.shape == (25, 3, 2)
    for k in range(3):
        for d in range(2):
            assert O.rel_l2(got[:, k, d], ref[:, k, d]) < 2e-5
    props = [O.propagator_tables(256, 256, spec.ax, spec.by, KEV, spec.cz / 40, precision="f64")] * 40
    P = O.probe(256, 256, spec.ax, spec.by, KEV, 0.0, k_ap, 0.0, 0.0, xy[:6], np.complex128)
    fp64 = O.stem(t.astype(np.complex128), props, seq, O.band_mask(256, 256, spec.ax, spec.by), P,
                  O.detector_masks(256, 256, spec.ax, spec.by, det), cps)
    for k in range(3):
        for d in range(2):
            assert O.rel_l2(got[:6, k, d], fp64[:, k, d]) < 1e-4


def test_resident_early_checkpoint_and_batches(ctx):
    """A last checkpoint before the last slice ends the loop there; the result
    does not depend on the probe batch."""
    from multislice_gb300 import Context
    spec, t, k_ap, det = _case(ctx)
    xy = S.raster(1.0, 3.0, 1.0, 3.0, 4, 3)
    seq = np.arange(40)
    full = ctx.stem_scan(t, spec.cz / 40, seq, spec.ax, spec.by, KEV, k_ap, xy, det, checkpoints=[5, 17],
                         resident=True)
    ref = ctx.stem_scan(t, spec.cz / 40, seq, spec.ax, spec.by, KEV, k_ap, xy, det, checkpoints=[5, 17])
    assert O.rel_l2(full, ref) < 2e-5
    with Context(0) as c:
        c.set_probe_batch(5)
        part = c.stem_scan(t, spec.cz / 40, seq, spec.ax, spec.by, KEV, k_ap, xy, det, checkpoints=[5, 17],
                           resident=True)
    assert np.array_equal(part, full)


def test_resident_rejects_other_sides(ctx):
    from multislice_gb300 import MslError
    t = np.ones((1, 128, 128), np.complex64)
    with pytest.raises(MslError) as e:
        ctx.stem_scan(t, 1.0, [0], 10.0, 10.0, KEV, 1.0, [[1.0, 1.0]], [(0.0, 1.0)], resident=True)
    assert e.value.code == -4
