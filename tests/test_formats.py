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
