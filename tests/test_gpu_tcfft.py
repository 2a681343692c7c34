"""The tensor-core form of the slice loop (schedule MSL_FAM_TC: line DFTs as
split-bf16 contractions on tcgen05) against the FP64 oracle: CTEM batches at
256^2 and 512^2 and the SrTiO3 512^2 STEM scan on a probe subset."""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu
TC = 3


@pytest.mark.parametrize("n", [256, 512])
def test_tc_multislice_matches_fp64(ctx, n):
    rng = np.random.default_rng(n + 1)
    t = np.exp(1j * 0.4 * rng.standard_normal((2, n, n))).astype(np.complex64)
    psi = (rng.standard_normal((3, n, n)) + 1j * rng.standard_normal((3, n, n))).astype(np.complex64)
    ax = by = 0.06 * n
    seq = [0, 1, 1, 0, 1]
    mask = O.band_mask(n, n, ax, by)
    props = [O.propagator_tables(n, n, ax, by, 200.0, 1.9, precision="f64")] * 2
    ref, _ = O.multislice(psi.astype(np.complex128), t.astype(np.complex128), props, seq, mask)
    ctx.set_schedule(n, TC, TC)
    try:
        got = ctx.multislice(t, 1.9, seq, ax, by, 200.0, psi=psi.copy())
    finally:
        ctx.set_schedule(n, 0, 0)
    fp32 = ctx.multislice(t, 1.9, seq, ax, by, 200.0, psi=psi.copy())
    e_tc, e_fp32 = O.rel_l2(got, ref), O.rel_l2(fp32, ref)
    assert e_tc < 1e-4, (e_tc, e_fp32)


def test_tc_stem_scan_subset_vs_fp64(ctx):
    """SrTiO3 8x8x50 cells, 512^2, 100 slices: 8 probes of the 64x64 raster."""
    import torch

    from multislice_gb300 import fparams_table
    from oracle import fp64_gpu
    cfg = S.config_srtio3_stem()
    spec = cfg["spec"]
    xy = cfg["probe_xy"][::512][:8]
    v = ctx.potential(spec, 512, 512, 100, cfg["radius"])
    t = ctx.transmission(v, spec.ax, spec.by, 200.0)
    ctx.set_schedule(512, TC, TC)
    try:
        got = ctx.stem_scan(t, spec.cz / 100, np.arange(100), spec.ax, spec.by, 200.0, cfg["k_ap"], xy,
                            cfg["det_k"], checkpoints=[49, 99])
    finally:
        ctx.set_schedule(512, 0, 0)
    dev = torch.device("cuda", 0)
    V = fp64_gpu.potential(spec.x, spec.y, spec.z, spec.Z, fparams_table(), spec.ax, spec.by, spec.cz, 512, 512,
                           100, cfg["radius"], dev)
    T = fp64_gpu.transmission(V, 200.0, spec.ax, spec.by)
    del V
    P = fp64_gpu.propagator(512, 512, spec.ax, spec.by, 200.0, spec.cz / 100, dev)
    ref = fp64_gpu.stem_scan(T, P, np.arange(100), 512, 512, spec.ax, spec.by, 200.0, cfg["k_ap"], xy,
                             cfg["det_k"], [49, 99], batch=8)
    del T
    torch.cuda.empty_cache()
    for k in range(2):
        for d in range(2):
            assert O.rel_l2(got[:, k, d], ref[:, k, d]) < 1e-3


def test_tc_schedule_rejected_on_other_sides(ctx):
    from multislice_gb300 import MslError
    with pytest.raises(MslError):
        ctx.set_schedule(1024, TC, TC)
    assert ctx.get_schedule(1024) == (0, 0)
