"""The C-ABI library loads without a GPU, exports every symbol include/msl.h
declares, and its host-only entry points agree with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from multislice_gb300 import _abi
from oracle import msl_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "msl.h")


def _lib():
    if not os.path.exists(_abi.LIB_PATH):
        from multislice_gb300 import build
        build.build()
    return ctypes.CDLL(_abi.LIB_PATH)


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(msl_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_binding_surface():
    assert set(declared_symbols()) == set(_abi.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = _lib()
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_host_constants_match_oracle():
    lib = _abi.load()
    for kev in (80.0, 200.0, 300.0):
        assert lib.msl_wavelength(kev) == pytest.approx(O.wavelength(kev), rel=1e-15)
        assert lib.msl_sigma(kev) == pytest.approx(O.sigma(kev), rel=1e-15)


def _fparams_text(tab):
    lines = []
    for z in range(1, 104):
        lines.append(f"Z={z:3d},  chisq=    0.100000")
        r = tab[z]
        for i in range(0, 12, 4):
            lines.append("  " + "  ".join(f"{v:.8e}" for v in r[i:i + 4]))
        lines.append("")
    return "\n".join(lines)


def test_fparams_parse_roundtrip(fparams):
    lib = _abi.load()
    text = _fparams_text(fparams).encode()
    out = np.zeros((104, 12), np.float64)
    rc = lib.msl_fparams_parse(text, len(text), out.ctypes.data)
    assert rc == 0
    np.testing.assert_allclose(out, fparams, rtol=1e-8)
    bad = text[: len(text) // 2]
    assert lib.msl_fparams_parse(bad, len(bad), out.ctypes.data) == _abi.MSL_E_ARG


def test_ctx_create_reports_missing_gpu_as_error():
    """Without a visible GPU the library refuses loudly instead of falling back."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    lib = _abi.load()
    h = ctypes.c_void_p()
    rc = lib.msl_ctx_create(0, ctypes.byref(h))
    assert rc in (_abi.MSL_E_CUDA, _abi.MSL_E_ARG)
    assert not h.value


def test_library_exports_muslib_entry_points():
    lib = _lib()
    text = open(HEADER).read()
    for name in _abi.MUSLIB_EXPORTS:
        assert hasattr(lib, name), name
        assert f"{name}(" in text


COO = """// SrTiO3 test cell
3.905 3.905 3.905 90 90 90 5

0.0 0.0 0.0 38 0.5
0.5 0.5 0.5 22
0.5 0.5 0.0 8 0 0.02 1
1.5 0.0 -0.5 8   // wrapped into [0, 1)
0.0 0.5 0.5 8 0.1 0.2 0.5
"""


def test_coo_parse_reference_rules():
    from multislice_gb300.specimen import parse_coo
    cell, rec = parse_coo(COO)
    assert (cell.a, cell.gamma, cell.natom) == (3.905, 90.0, 5)
    np.testing.assert_allclose(rec[0], [0, 0, 0, 38, 0.5, 0, 1])
    np.testing.assert_allclose(rec[1], [0.5, 0.5, 0.5, 22, 0, 0, 1])
    np.testing.assert_allclose(rec[3][:3], [0.5, 0.0, 0.5])
    np.testing.assert_allclose(rec[4], [0, 0.5, 0.5, 8, 0.1, 0.2, 0.5])
    # amodel style: a title line before the header
    cell2, rec2 = parse_coo("Fe model\n2.87 2.87 2.87 90 90 90 1\n0.25 0.25 0.25 26\n")
    assert cell2.natom == 1 and rec2[0][3] == 26
    with pytest.raises(Exception):
        parse_coo("1 2 3 90 90 90 4\n0 0 0 8\n")  # fewer records than declared


def test_coo_roundtrip(tmp_path):
    from multislice_gb300 import specimen as S
    spec = S.srtio3(2, 2, 2)
    p = tmp_path / "sto.coo"
    S.write_coo(spec, str(p), "SrTiO3 2x2x2")
    back = S.read_coo(str(p))
    np.testing.assert_allclose(back.x, spec.x, atol=1e-9)
    np.testing.assert_allclose(back.z, spec.z, atol=1e-9)
    assert np.array_equal(back.Z, spec.Z) and back.cz == spec.cz
