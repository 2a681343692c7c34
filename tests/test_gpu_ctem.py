"""GPU parity of the CTEM imaging epilogue and the frozen-phonon driver
(objective lens of mulslice.cpp:539-676, jitter of MSUseOnceCalculator.cs:179-199)."""
import numpy as np
import pytest

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu

CS = 1.2e7      # 1.2 mm in Angstrom
DF = -600.0     # -60 nm


def test_vacuum_image_is_uniform(ctx):
    """A plane wave through vacuum images to intensity 1 everywhere (CTF(0) = 1)."""
    t = np.ones((1, 128, 128), np.complex64)
    img, psi, ex = ctx.ctem_image(t, 2.0, [0] * 4, 20.0, 20.0, 300.0, CS, DF, 2.0,
                                  exit_intensity=np.zeros((128, 128)))
    np.testing.assert_allclose(img, 1.0, atol=1e-6)
    np.testing.assert_allclose(ex, 1.0, atol=1e-6)
    img2, _, _ = ctx.ctem_image(t, 2.0, [0] * 4, 20.0, 20.0, 300.0, CS, DF, 2.0, df_spread=50.0,
                                df_step=25.0)
    np.testing.assert_allclose(img2, 1.0, atol=1e-6)


@pytest.mark.parametrize("spread", [0.0, 50.0])
def test_ctem_image_vs_oracle(ctx, golden, spread):
    G = golden("si_small.npz")
    ax, by, dz = float(G["ax"]), float(G["by"]), float(G["dz"])
    img, psi, _ = ctx.ctem_image(G["t"], dz, G["seq"], ax, by, 200.0, CS, DF, 1.5,
                                 df_spread=spread, df_step=25.0)
    assert O.rel_l2(psi[0], G["wave"]) < 1e-5          # exit wave vs the reference
    ref = O.ctem_image(G["wave"].astype(np.complex128), ax, by, 200.0, CS, DF, 1.5, spread, 25.0)
    assert O.rel_l2(img, ref) < 2e-5


def _oracle_frozen_phonon(spec, fp, nx, ny, nslice, radius, kev, k_obj, nconfig, sigma, seed):
    img = np.zeros((nx, ny))
    exi = np.zeros((nx, ny))
    mask = O.band_mask(nx, ny, spec.ax, spec.by)
    props = [O.propagator_tables(nx, ny, spec.ax, spec.by, kev, spec.cz / nslice, precision="f64")]
    for c in range(nconfig):
        d = O.phonon_displacements(seed, c, spec.natom, sigma)
        V = O.potential(spec.x + d[:, 0], spec.y + d[:, 1], spec.z + d[:, 2], spec.Z, fp, spec.ax,
                        spec.by, spec.cz, nx, ny, nslice, radius)
        T = O.transmission(V, kev, spec.ax, spec.by, np.complex128)
        w, _ = O.multislice(np.ones((nx, ny), np.complex128), T, props * nslice, np.arange(nslice), mask)
        img += O.ctem_image(w, spec.ax, spec.by, kev, CS, DF, k_obj) / nconfig
        exi += np.abs(w) ** 2 / nconfig
    return img, exi


def test_frozen_phonon_vs_oracle(ctx, fparams):
    spec = S.fcc_au(2, 2, 4)
    nx = ny = 128
    img, exi = ctx.frozen_phonon(spec, nx, ny, 8, 3.0, 300.0, CS, DF, 2.0, nconfig=3, sigma=0.085,
                                 seed=7)
    ref_img, ref_exi = _oracle_frozen_phonon(spec, fparams, nx, ny, 8, 3.0, 300.0, 2.0, 3, 0.085, 7)
    assert O.rel_l2(exi, ref_exi) < 2e-5
    assert O.rel_l2(img, ref_img) < 2e-5


def test_frozen_phonon_batch_size_does_not_change_the_average():
    """Configurations run in batches through one slice loop; a memory cap that
    leaves room for one configuration per batch gives bit-identical averages."""
    from multislice_gb300 import Context
    spec = S.fcc_au(2, 2, 4)
    args = (spec, 128, 128, 8, 3.0, 300.0, CS, DF, 2.0)
    with Context(0) as c:
        l0 = c.launches
        img_b, exi_b = c.frozen_phonon(*args, nconfig=5, sigma=0.085, seed=11)
        batched = c.launches - l0
    with Context(0) as c:
        # transmissions of one configuration: 1 MiB; a 4 MiB cap leaves a 2 MiB
        # batch budget, so one configuration per batch
        c.set_memory_limit(4 << 20)
        l0 = c.launches
        img_1, exi_1 = c.frozen_phonon(*args, nconfig=5, sigma=0.085, seed=11)
        single = c.launches - l0
        assert c.memory_in_use() <= 4 << 20
    assert single > batched   # five slice loops instead of one
    assert np.array_equal(img_b, img_1)
    assert np.array_equal(exi_b, exi_1)


def test_frozen_phonon_zero_sigma_equals_static_image(ctx):
    spec = S.fcc_au(2, 2, 4)
    img, exi = ctx.frozen_phonon(spec, 128, 128, 8, 3.0, 300.0, CS, DF, 2.0, nconfig=2, sigma=0.0, seed=1)
    v = ctx.potential(spec, 128, 128, 8, 3.0)
    t = ctx.transmission(v, spec.ax, spec.by, 300.0)
    ref, _, _ = ctx.ctem_image(t, spec.cz / 8, np.arange(8), spec.ax, spec.by, 300.0, CS, DF, 2.0)
    assert O.rel_l2(img, ref) < 1e-6


def test_frozen_phonon_au_2048_full_size(ctx):
    """fcc Au 16x16x40 cells, 2048^2, 80 slices, 32 configurations, 300 kV, Cs 1.2 mm,
    df -60 nm: configuration averaging is deterministic, physically bounded and,
    on every pixel, within 1e-4 of the FP64 oracle."""
    spec = S.fcc_au()
    kev = 300.0
    k_obj = float(S.mrad_to_k(25.0, kev))
    img, exi = ctx.frozen_phonon(spec, 2048, 2048, 80, 3.0, kev, CS, DF, k_obj, nconfig=32,
                                 sigma=0.085, seed=2026)
    assert np.all(np.isfinite(img)) and np.all(img >= 0)
    assert 0.5 < exi.mean() <= 1.0 + 1e-6          # band limiting only removes intensity
    assert img.mean() <= exi.mean() + 1e-6          # the aperture only removes intensity
    img2, _ = ctx.frozen_phonon(spec, 2048, 2048, 80, 3.0, kev, CS, DF, k_obj, nconfig=32,
                                sigma=0.085, seed=2026, want_exit=False)
    assert np.array_equal(img, img2)
    # every pixel against the FP64 oracle (torch complex128 on the same GPU), same seed
    import torch

    from oracle import fp64_gpu
    from multislice_gb300 import fparams_table
    ref_img, ref_exi = fp64_gpu.frozen_phonon(spec, fparams_table(), 2048, 2048, 80, 3.0, kev, CS, DF, k_obj,
                                              32, 0.085, 2026, torch.device("cuda", 0))
    torch.cuda.empty_cache()
    assert O.rel_l2(exi, ref_exi) < 1e-4
    assert O.rel_l2(img, ref_img) < 1e-4


def test_astigmatic_image_vs_oracle(ctx, golden):
    G = golden("si_small.npz")
    ax, by, dz = float(G["ax"]), float(G["by"]), float(G["dz"])
    astig = (40.0, 0.3, 300.0, -0.7)
    img, psi, _ = ctx.ctem_image(G["t"], dz, G["seq"], ax, by, 200.0, CS, DF, 1.5, astig=astig)
    ref = O.ctem_image(G["wave"].astype(np.complex128), ax, by, 200.0, CS, DF, 1.5, astig=astig)
    assert O.rel_l2(img, ref) < 2e-5


def test_partial_coherence_vs_oracle(ctx, golden):
    G = golden("si_small.npz")
    ax, by, dz = float(G["ax"]), float(G["by"]), float(G["dz"])
    acmax = 0.005                       # 5 mrad condenser: 13 angles in this 10.9 A cell
    img, na = ctx.partial_coherence(G["t"], dz, G["seq"], ax, by, 200.0, CS, DF, 1.5, 0.0, acmax,
                                    df_spread=40.0, df_step=20.0, astig=(20.0, 0.1, 0.0, 0.0))
    mask = O.band_mask(64, 64, ax, by)
    props = [O.propagator_tables(64, 64, ax, by, 200.0, dz, precision="f64")] * 8
    ref, nref = O.partial_coherence(G["t"].astype(np.complex128), props, G["seq"], mask, ax, by, 200.0,
                                    CS, DF, 1.5, 0.0, acmax, 40.0, 20.0, (20.0, 0.1, 0.0, 0.0))
    assert na == nref and na > 1
    assert O.rel_l2(img, ref) < 2e-5


def test_partial_coherence_single_angle_equals_coherent_image(ctx, golden):
    """With the condenser closed to the axis only the untilted wave remains."""
    G = golden("si_small.npz")
    ax, by, dz = float(G["ax"]), float(G["by"]), float(G["dz"])
    img, na = ctx.partial_coherence(G["t"], dz, G["seq"], ax, by, 200.0, CS, DF, 1.5, 0.0, 0.0,
                                    df_spread=30.0, df_step=15.0)
    ref, _, _ = ctx.ctem_image(G["t"], dz, G["seq"], ax, by, 200.0, CS, DF, 1.5, df_spread=30.0,
                               df_step=15.0)
    assert na == 1
    assert O.rel_l2(img, ref) < 1e-6


# ------------------------------------------- against the compiled reference's images
# tests/golden/ctem_partial.npz: mulslice.cpp:539-676 (partial coherence, defocus
# spread, objective aperture, 2- and 3-fold astigmatism) driven by the reference's
# own cfpix transforms and propagate() (tests/golden/make_ctem_golden.py).

def _lens(G, ci, lam):
    acmin, acmax, cs, df0, sigf, dfd, aobj, dfa2, dfa2p, dfa3, dfa3p = G["cases"][ci]
    return dict(acmin=acmin * 1e-3, acmax=acmax * 1e-3, cs=cs * 1e7, df=df0, df_spread=sigf, df_step=dfd,
                k_obj=float(np.float32(aobj * 1e-3) / np.float32(lam)),
                astig=(dfa2, np.radians(dfa2p), dfa3, np.radians(dfa3p)))


@pytest.mark.parametrize("ci", [0, 1, 2])
def test_partial_coherence_vs_compiled_reference(ctx, golden, ci):
    G = golden("ctem_partial.npz")
    S = golden("si_small.npz")
    ax, by, dz, kev = float(S["ax"]), float(S["by"]), float(S["dz"]), float(S["kev"])
    L = _lens(G, ci, float(np.float32(O.wavelength(kev))))
    img, nang = ctx.partial_coherence(S["t"], dz, S["seq"], ax, by, kev, L["cs"], L["df"], L["k_obj"],
                                      L["acmin"], L["acmax"], df_spread=L["df_spread"], df_step=L["df_step"],
                                      astig=L["astig"])
    assert nang == int(G[f"pc_{ci}_nillum"])
    assert O.rel_l2(img, G[f"pc_{ci}_pix"]) < 2e-5


@pytest.mark.parametrize("ci", [1, 2])
def test_ctem_image_vs_compiled_reference(ctx, golden, ci):
    """One illumination angle: msl_ctem_image's lens with the reference's image."""
    G = golden("ctem_partial.npz")
    S = golden("si_small.npz")
    ax, by, dz, kev = float(S["ax"]), float(S["by"]), float(S["dz"]), float(S["kev"])
    L = _lens(G, ci, float(np.float32(O.wavelength(kev))))
    img, _, _ = ctx.ctem_image(S["t"], dz, S["seq"], ax, by, kev, L["cs"], L["df"], L["k_obj"],
                               df_spread=L["df_spread"], df_step=L["df_step"], astig=L["astig"])
    assert O.rel_l2(img, G[f"pc_{ci}_pix"]) < 2e-5
