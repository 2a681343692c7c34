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
