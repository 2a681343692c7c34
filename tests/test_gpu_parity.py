"""GPU parity: libmsl.so (through the C ABI) against the reference's golden vectors
and the oracle.  Tolerances are relative L2 norms: 1e-4 on exit waves and 1e-3
on STEM images are the required bars; the tighter numbers below are what the
FP32 path actually holds and guard against regressions."""
import numpy as np
import pytest

from multislice_gb300 import MslError, specimen as S
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu

SIDES = [64, 128, 256, 384, 512, 768, 1024, 2048]


def rand_c64(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("n", SIDES)
def test_fft2d_matches_direct_transform(ctx, n):
    rng = np.random.default_rng(n)
    x = rand_c64(rng, (2, n, n))
    ref = O.kfft(x.astype(np.complex128))
    got = ctx.fft2d(x.copy(), 10.0, 10.0, +1)
    assert O.rel_l2(got, ref) < 3e-6
    back = ctx.fft2d(got.copy(), 10.0, 10.0, -1)
    assert O.rel_l2(back, x) < 3e-6


def test_fft2d_non_square(ctx):
    rng = np.random.default_rng(5)
    x = rand_c64(rng, (3, 256, 512))
    got = ctx.fft2d(x.copy(), 10.0, 20.0, +1)
    assert O.rel_l2(got, O.kfft(x.astype(np.complex128))) < 3e-6
    got = ctx.fft2d(x.copy(), 10.0, 20.0, -1)
    assert O.rel_l2(got, O.kifft(x.astype(np.complex128))) < 3e-6


def test_potential_small_vs_reference(ctx, golden):
    G = golden("si_small.npz")
    spec = S.si_diamond(2, 2, 2, 5.431)
    v = ctx.potential(spec, 64, 64, 8, 3.0)
    assert O.rel_l2(v, G["v"]) < 2e-6
    assert np.abs(v - G["v"]).max() < 1e-5 * np.abs(G["v"]).max()


def test_potential_config1_vs_reference(ctx, golden):
    C = golden("si_config1.npz")
    cfg = S.config_si_ctem()
    v = ctx.potential(cfg["spec"], 256, 256, 80, cfg["radius"]).astype(np.float64)
    np.testing.assert_allclose([v.sum(), (v ** 2).sum()], C["v_checksum"], rtol=2e-6)
    assert O.rel_l2(v[0], C["v0"]) < 2e-6


def test_potential_empty_and_outside_atoms(ctx):
    spec = S.Specimen(np.array([1.0]), np.array([1.0]), np.array([50.0]), np.array([14], np.int32),
                      20.0, 20.0, 10.0)
    v = ctx.potential(spec, 64, 64, 4, 3.0)
    assert np.all(v == 0)
    empty = S.Specimen(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0, np.int32), 20.0, 20.0, 10.0)
    assert np.all(ctx.potential(empty, 64, 64, 2, 3.0) == 0)


@pytest.mark.parametrize("natom", [300, 513, 1500])
def test_potential_dense_slices_vs_oracle(ctx, fparams, natom):
    """A slice holding fewer and more atoms than the gather keeps in shared memory
    (512), with tiles that keep more than one list of 64 atoms, and an empty
    slice after it: equal to the FP64 oracle within FP32 rounding."""
    rng = np.random.default_rng(natom)
    a = 16.0
    x, y = rng.uniform(0, a, natom), rng.uniform(0, a, natom)
    z = rng.uniform(0, 1.5, natom)                  # all in the first of two 1.5 A slices
    Z = rng.choice([6, 14, 29, 79], natom).astype(np.int32)
    spec = S.Specimen(x, y, z, Z, a, a, 3.0)
    v = ctx.potential(spec, 128, 128, 2, 2.5).astype(np.float64)
    ref = O.potential(x, y, z, Z, fparams, a, a, 3.0, 128, 128, 2, 2.5)
    assert O.rel_l2(v, ref) < 2e-6


def test_transmission_small_vs_reference(ctx, golden):
    G = golden("si_small.npz")
    t = ctx.transmission(G["v"].astype(np.float32), float(G["ax"]), float(G["by"]), 200.0)
    assert O.rel_l2(t, G["t"]) < 2e-6


def test_ctem_small_vs_reference(ctx, golden):
    G = golden("si_small.npz")
    w = ctx.multislice(G["t"], float(G["dz"]), G["seq"], float(G["ax"]), float(G["by"]), 200.0)
    assert O.rel_l2(w[0], G["wave"]) < 1e-5


def test_ctem_config1_end_to_end_vs_reference(ctx, golden, fparams):
    """Si 256^2, 80 slices: GPU potential -> transmission -> slice loop vs Kirkland's mulslice."""
    C = golden("si_config1.npz")
    cfg = S.config_si_ctem()
    spec = cfg["spec"]
    v = ctx.potential(spec, 256, 256, 80, cfg["radius"])
    t = ctx.transmission(v, spec.ax, spec.by, 200.0)
    w = ctx.multislice(t, spec.cz / 80, np.arange(80), spec.ax, spec.by, 200.0)[0]
    err = O.rel_l2(w, C["wave"])
    assert err < 1e-4, err          # the required bar
    assert err < 2e-5, err          # what the path holds


def test_ctem_batch_of_entrance_waves(ctx, golden):
    G = golden("si_small.npz")
    rng = np.random.default_rng(2)
    ax, by = float(G["ax"]), float(G["by"])
    psi = rand_c64(rng, (3, 64, 64))
    got = ctx.multislice(G["t"], float(G["dz"]), G["seq"], ax, by, 200.0, psi=psi.copy())
    mask = O.band_mask(64, 64, ax, by)
    props = [O.propagator_tables(64, 64, ax, by, 200.0, float(G["dz"]), precision="f64")] * 8
    ref, _ = O.multislice(psi.astype(np.complex128), G["t"].astype(np.complex128), props, G["seq"], mask)
    assert O.rel_l2(got, ref) < 1e-5


def test_ctem_vacuum_keeps_plane_wave(ctx):
    t = np.ones((2, 128, 128), np.complex64)
    w = ctx.multislice(t, 2.0, [0, 1, 0, 1], 20.0, 20.0, 300.0)
    np.testing.assert_allclose(w, 1.0, atol=1e-6)


def _stem_small_inputs(G):
    return (float(G["ax"]), float(G["by"]), float(G["kev"]), float(G["dz"]))


def test_stem_small_vs_reference(ctx, golden):
    G = golden("stem_small.npz")
    ax, by, kev, dz = _stem_small_inputs(G)
    t = ctx.transmission(G["v"], ax, by, kev)
    d = ctx.stem_scan(t, dz, np.arange(20), ax, by, kev, float(G["k_ap"]), G["xy"], G["det_k"],
                      checkpoints=list(G["cps"]))
    assert d.shape == G["det"].shape
    assert O.rel_l2(d, G["det"]) < 1e-5
    for k in range(d.shape[-1]):
        assert O.rel_l2(d[..., k], G["det"][..., k]) < 1e-4


def test_stem_batching_is_invisible(ctx, golden):
    G = golden("stem_small.npz")
    ax, by, kev, dz = _stem_small_inputs(G)
    t = ctx.transmission(G["v"], ax, by, kev)
    args = (t, dz, np.arange(20), ax, by, kev, float(G["k_ap"]), G["xy"], G["det_k"])
    ctx.set_probe_batch(16)
    a = ctx.stem_scan(*args, checkpoints=[19])
    ctx.set_probe_batch(3)
    b = ctx.stem_scan(*args, checkpoints=[19])
    ctx.set_probe_batch(0)
    assert np.array_equal(a, b)


def test_stem_vacuum_known_answer(ctx):
    """In vacuum |Psi(k)|^2 is 1 on every aperture pixel: a detector over all k
    counts the aperture pixels, one outside the aperture sees nothing."""
    n, a, kev = 256, 25.0, 200.0
    k_ap = float(S.mrad_to_k(20.0, kev))
    t = np.ones((1, n, n), np.complex64)
    xy = np.array([[3.3, 7.1], [12.5, 12.5]])
    det = [(0.0, 50.0), (2.0 * k_ap, 3.0 * k_ap)]
    d = ctx.stem_scan(t, 2.0, [0] * 5, a, a, kev, k_ap, xy, det)
    kx, ky = O.k_tables_f64(n, n, a, a)
    s = kx[:, None] ** 2 + ky[None, :] ** 2
    n_ap = int((s <= k_ap ** 2).sum())
    np.testing.assert_allclose(d[:, 0, 0], n_ap, rtol=1e-5)
    assert np.all(np.abs(d[:, 0, 1]) < 1e-6 * n_ap)


def test_stem_config2_subset_vs_reference(ctx, golden):
    """SrTiO3 512^2, 100 slices, 8 raster probes: full GPU chain vs the reference."""
    C = golden("stem_config2.npz")
    cfg = S.config_srtio3_stem()
    spec = cfg["spec"]
    v = ctx.potential(spec, 512, 512, 100, cfg["radius"])
    np.testing.assert_allclose([v.astype(np.float64).sum()], C["v_checksum"][:1], rtol=2e-6)
    t = ctx.transmission(v, spec.ax, spec.by, 200.0)
    d = ctx.stem_scan(t, spec.cz / 100, np.arange(100), spec.ax, spec.by, 200.0, cfg["k_ap"],
                      C["xy"], cfg["det_k"])
    for k in range(2):  # HAADF, ABF images
        err = O.rel_l2(d[:, 0, k], C["det"][:, 0, k])
        assert err < 1e-3, err   # the required bar
        assert err < 5e-5, err   # what the path holds


def test_stem_config2_full_image_vs_fp64(ctx):
    """The whole 64x64-probe HAADF and ABF images of the SrTiO3 512^2, 100-slice
    scan against the FP64 oracle (torch complex128 on the same GPU, potential
    included): the 1e-3 bar of the metric on every pixel."""
    import torch

    from multislice_gb300 import fparams_table
    from oracle import fp64_gpu
    cfg = S.config_srtio3_stem()
    spec = cfg["spec"]
    v = ctx.potential(spec, 512, 512, 100, cfg["radius"])
    t = ctx.transmission(v, spec.ax, spec.by, 200.0)
    d = ctx.stem_scan(t, spec.cz / 100, np.arange(100), spec.ax, spec.by, 200.0, cfg["k_ap"],
                      cfg["probe_xy"], cfg["det_k"])
    dev = torch.device("cuda", 0)
    V = fp64_gpu.potential(spec.x, spec.y, spec.z, spec.Z, fparams_table(), spec.ax, spec.by, spec.cz, 512, 512,
                           100, cfg["radius"], dev)
    T = fp64_gpu.transmission(V, 200.0, spec.ax, spec.by)
    del V
    P = fp64_gpu.propagator(512, 512, spec.ax, spec.by, 200.0, spec.cz / 100, dev)
    ref = fp64_gpu.stem_scan(T, P, np.arange(100), 512, 512, spec.ax, spec.by, 200.0, cfg["k_ap"],
                             cfg["probe_xy"], cfg["det_k"], [99], batch=256)
    del T
    torch.cuda.empty_cache()
    for k in range(2):
        err = O.rel_l2(d[:, 0, k], ref[:, 0, k])
        assert err < 1e-3, err   # the metric's bar
        assert err < 1e-4, err   # what the path holds


def test_invalid_arguments_fail_before_launch(ctx):
    t = np.ones((1, 100, 100), np.complex64)
    with pytest.raises(MslError) as e:
        ctx.multislice(t, 1.0, [0], 10.0, 10.0, 200.0)
    assert e.value.code == -4
    t = np.ones((1, 64, 64), np.complex64)
    with pytest.raises(MslError):
        ctx.multislice(t, 1.0, [1], 10.0, 10.0, 200.0)       # layer index out of range
    with pytest.raises(MslError):
        ctx.multislice(t, -1.0, [0], 10.0, 10.0, 200.0)      # negative thickness
    with pytest.raises(MslError):
        ctx.stem_scan(t, 1.0, [0], 10.0, 10.0, 200.0, 1.0, [[np.nan, 0.0]], [(0.0, 1.0)])
    with pytest.raises(MslError):
        ctx.stem_scan(t, 1.0, [0], 10.0, 10.0, 200.0, 1.0, [[0.0, 0.0]], [(0.0, 1.0)],
                      checkpoints=[3])
    spec = S.Specimen(np.array([1.0]), np.array([1.0]), np.array([1.0]), np.array([0], np.int32),
                      20.0, 20.0, 10.0)
    with pytest.raises(MslError):
        ctx.potential(spec, 64, 64, 4, 3.0)                  # Z = 0
    spec.Z[:] = 6
    with pytest.raises(MslError):
        ctx.potential(spec, 64, 64, 4, 10.0)                 # radius >= half the cell
    # the context is still usable
    w = ctx.multislice(t, 1.0, [0], 10.0, 10.0, 200.0)
    assert np.allclose(w, 1.0, atol=1e-6)


def test_device_buffers_match_host_buffers(ctx, golden):
    torch = pytest.importorskip("torch")
    G = golden("stem_small.npz")
    ax, by, kev, dz = _stem_small_inputs(G)
    v_host = G["v"].astype(np.float32)
    t_host = ctx.transmission(v_host, ax, by, kev)
    v_dev = torch.from_numpy(v_host).cuda()
    t_dev = torch.empty(v_host.shape + (2,), dtype=torch.float32, device="cuda")
    ctx.transmission(v_dev, ax, by, kev, out=t_dev)
    t_back = t_dev.cpu().numpy()
    assert np.array_equal(t_back[..., 0] + 1j * t_back[..., 1], t_host)
    out_dev = torch.empty((len(G["xy"]), 1, 3), dtype=torch.float64, device="cuda")
    ctx.stem_scan(t_dev, dz, np.arange(20), ax, by, kev, float(G["k_ap"]), G["xy"], G["det_k"],
                  out=out_dev)
    d_host = ctx.stem_scan(t_host, dz, np.arange(20), ax, by, kev, float(G["k_ap"]), G["xy"],
                           G["det_k"])
    assert np.array_equal(out_dev.cpu().numpy(), d_host)


def test_bounded_wait_reports_timeout_and_context_survives(ctx):
    """A wait that nothing completes gives up, raises the error flag, and leaves the
    context usable (failure detection without a GPU fault)."""
    assert ctx._lib.msl_check_wait_timeout(ctx._h, 256) == 0
    t = np.ones((1, 64, 64), np.complex64)
    w = ctx.multislice(t, 1.0, [0, 0], 10.0, 10.0, 200.0)
    np.testing.assert_allclose(w, 1.0, atol=1e-6)
