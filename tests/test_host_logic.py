"""Host-side logic: specimen generators, scan geometry, slice binning."""
import numpy as np

from multislice_gb300 import specimen as S
from oracle import msl_oracle as O


def test_si_diamond_counts_and_sites():
    s = S.si_diamond()
    assert s.natom == 8 * 5 * 5 * 20 == 4000
    assert np.all(s.Z == 14)
    assert np.isclose(s.ax, 27.155) and np.isclose(s.cz, 108.62)
    # every atom is centred in one a/4 slice
    kz = O.slice_index(s.z, s.cz, 80)
    frac = s.z / (s.cz / 80) - kz
    assert np.all(kz >= 0) and np.allclose(frac, 0.5)
    assert np.bincount(kz, minlength=80).tolist() == [50] * 80


def test_srtio3_counts_and_stoichiometry():
    s = S.srtio3()
    assert s.natom == 5 * 8 * 8 * 50 == 16000
    zc = np.bincount(s.Z)
    assert zc[38] == 3200 and zc[22] == 3200 and zc[8] == 9600
    kz = O.slice_index(s.z, s.cz, 100)
    assert np.all(kz >= 0)
    assert np.allclose(s.z / (s.cz / 100) - kz, 0.5)


def test_fcc_au_and_jitter_are_seeded():
    s = S.fcc_au(2, 2, 2)
    assert s.natom == 32
    a = S.jitter(s, 0.085, np.random.default_rng(7))
    b = S.jitter(s, 0.085, np.random.default_rng(7))
    assert np.array_equal(a.x, b.x)
    d = np.concatenate([a.x - s.x, a.y - s.y, a.z - s.z])
    assert 0.05 < d.std() < 0.12


def test_amorphous_min_separation():
    rng = np.random.default_rng(3)
    s = S.amorphous((20.0, 20.0), 10.0, 0.05, 1.5, [6, 14, 29, 79], [0.4, 0.3, 0.2, 0.1], rng)
    assert abs(s.natom - 200) <= 20
    p = np.stack([s.x, s.y, s.z], 1)
    d = p[:, None, :] - p[None, :, :]
    d[..., :2] -= np.round(d[..., :2] / 20.0) * 20.0
    r = np.sqrt((d ** 2).sum(-1)) + np.eye(len(p)) * 10
    assert r.min() >= 1.5 - 1e-9


def test_stem_raster_and_angles():
    cfg = S.config_srtio3_stem()
    xy = cfg["probe_xy"]
    assert xy.shape == (4096, 2)
    a = 3.905
    assert xy[:, 0].min() == 3 * a and xy[:, 0].max() < 5 * a
    lam = O.wavelength(200.0)
    assert np.isclose(cfg["k_ap"], 0.025 / lam)
    assert np.isclose(cfg["det_k"][0][1], 0.2 / lam)


def test_slice_index_drops_outside():
    kz = O.slice_index(np.array([-0.1, 0.0, 1.99, 2.0, 10.0]), 2.0, 4)
    assert kz.tolist() == [-1, 0, 3, -1, -1]


def test_phonon_displacement_stream_matches_oracle():
    from multislice_gb300 import phonon_displacements
    for seed, cfg, n in ((0, 0, 1), (1234, 5, 1000), (2 ** 63 + 11, 31, 40960)):
        a = phonon_displacements(seed, cfg, n, 0.085)
        b = O.phonon_displacements(seed, cfg, n, 0.085)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-15)
    d = phonon_displacements(99, 3, 40960, 0.085)
    assert abs(d.std() - 0.085) < 0.002 and abs(d.mean()) < 0.002
    assert not np.allclose(phonon_displacements(99, 4, 10, 0.085), phonon_displacements(99, 3, 10, 0.085))


def test_defocus_weights_follow_mulslice_rule():
    dfs, w = O.defocus_weights(-600.0, 50.0, 25.0)
    assert len(dfs) == 11 and np.isclose(w.sum(), 1.0)
    assert np.isclose(dfs[5], -600.0) and w[5] == w.max()


def test_uneven_jobs_follow_the_workload_rules():
    from multislice_gb300 import specimen as S
    a = S.uneven_jobs(11, 6, max_slices=30, max_box=30.0)
    b = S.uneven_jobs(11, 6, max_slices=30, max_box=30.0)
    for x, y in zip(a, b):                       # seeded
        assert (x["n"], x["nslice"], x["kev"]) == (y["n"], y["nslice"], y["kev"])
        assert np.array_equal(x["spec"].x, y["spec"].x)
    for j in a:
        assert j["n"] in (256, 384, 512, 768, 1024) and 20 <= j["nslice"] <= 30 and 1 <= j["dz"] <= 2
        s = j["spec"]
        vol = s.ax * s.by * s.cz
        assert abs(s.natom / vol - 0.05) < 0.005 and set(np.unique(s.Z)) <= {6, 14, 29, 79}
