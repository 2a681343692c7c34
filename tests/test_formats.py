"""On-disk formats and job files on the host: MRC round trip, job-file parsing rules."""
import numpy as np

from multislice_gb300 import jobs
from multislice_gb300.mrc import read_mrc, write_mrc


def test_mrc_roundtrip_float_and_complex(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((3, 16, 8)).astype(np.float32)
    write_mrc(tmp_path / "a.mrc", a, (10.0, 20.0, 5.0), ["potential"])
    b, h = read_mrc(tmp_path / "a.mrc")
    assert np.array_equal(a, b) and h["mode"] == 2 and h["labels"] == ["potential"]
    assert np.allclose(h["cell"], (10.0, 20.0, 5.0))
    c = (rng.standard_normal((16, 8)) + 1j * rng.standard_normal((16, 8))).astype(np.complex64)
    write_mrc(tmp_path / "c.mrc", c)
    d, h = read_mrc(tmp_path / "c.mrc")
    assert np.array_equal(c, d[0]) and h["mode"] == 4
    raw = open(tmp_path / "c.mrc", "rb").read()
    assert raw[208:212] == b"MAP " and len(raw) == 1024 + c.nbytes


def test_thickness_checkpoints_follow_the_csharp_rule():
    seq, cps = jobs._slices_to([6.14, 7.6, 47.0], 1.0, 4)
    assert cps == [6, 7, 46]              # first slice whose bottom reaches each thickness
    assert len(seq) == 47 and seq[:6].tolist() == [0, 1, 2, 3, 0, 1]


def test_csharp_wav_and_stem_roundtrip(tmp_path):
    from multislice_gb300.csfiles import read_stem, read_wav, write_stem, write_wav
    rng = np.random.default_rng(1)
    psi = (rng.standard_normal((8, 6)) + 1j * rng.standard_normal((8, 6))).astype(np.complex64)
    write_wav(tmp_path / "w.wav", psi, 31.24, 30.0, 195.25, 200.0)
    raw = open(tmp_path / "w.wav", "rb").read()
    assert len(raw) == 8 * 6 * 16 + 160 and raw[-160:].startswith(b"___ ")
    # the C# layout: row j (y) major, conjugate convention
    first = np.frombuffer(raw[:16], dtype=np.complex128)[0]
    assert first == np.conj(psi[0, 0]) and np.frombuffer(raw[16:32], np.complex128)[0] == np.conj(psi[1, 0])
    back, meta = read_wav(tmp_path / "w.wav")
    assert np.array_equal(back, psi.astype(np.complex128))
    assert (meta["n"], meta["m"], meta["kev"]) == (8, 6, 200.0) and abs(meta["thickness"] - 195.25) < 1e-9
    img = rng.random((4, 3))
    write_stem(tmp_path / "s.stem", img, (0.6, 0.4), 15.62, 200.0)
    back, meta = read_stem(tmp_path / "s.stem")
    assert np.array_equal(back, img) and (meta["n"], meta["m"]) == (4, 3)


def test_csharp_cbed_slice_and_slice_coo(tmp_path):
    from multislice_gb300 import csfiles as C
    rng = np.random.default_rng(2)
    n, m = 8, 6
    spec = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
    C.write_cbed(tmp_path / "d.cbed", spec, 10.0, 12.0, 50.0, 300.0)
    raw = open(tmp_path / "d.cbed", "rb").read()
    assert len(raw) == n * m * 8 + 160 and raw[-160:].startswith(b"~~~ ")
    out = np.frombuffer(raw[: n * m * 8], np.float64).reshape(m, n)
    # zero frequency at (row M/2, column N/2), as MSProject.cs:658-667 writes it
    assert out[m // 2, n // 2] == abs(spec[0, 0]) ** 2
    assert out[0, 0] == abs(spec[n // 2, m // 2]) ** 2
    assert out[m // 2, n // 2 + 1] == abs(spec[1, 0]) ** 2
    back, meta = C.read_cbed(tmp_path / "d.cbed")
    assert np.array_equal(back, np.abs(spec) ** 2) and meta["kev"] == 300.0
    t = np.exp(1j * rng.standard_normal((n, m))).astype(np.complex64)
    C.write_slice(tmp_path / "s.slice", t, 3.905, 3.905, 1.9525, 7, 100, nmult=8, mmult=8)
    tb, meta = C.read_slice(tmp_path / "s.slice")
    assert np.array_equal(tb, t.astype(np.complex128))
    assert meta["kev"] == -1.0 and meta["f9"] == 7 and meta["f10"] == 100 and abs(meta["a"] - 31.24) < 1e-9
    atoms = {"x": rng.random(5), "y": rng.random(5), "z": rng.random(5) * 2, "DW": rng.random(5),
             "ads": rng.random(5) * 0.1, "occ": np.ones(5), "type": np.arange(5, dtype=np.int32),
             "type_": np.array([8, 8, 22, 38, 8], np.int32)}
    C.write_slice_coo(tmp_path / "a.slice_coo", 1.9525, atoms)
    assert len(open(tmp_path / "a.slice_coo", "rb").read()) == 4 + 8 + 5 * (6 * 8 + 2 * 4)
    th, back = C.read_slice_coo(tmp_path / "a.slice_coo")
    assert th == 1.9525 and all(np.array_equal(back[k], atoms[k]) for k in atoms)
