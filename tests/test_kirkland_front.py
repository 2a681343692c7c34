"""Kirkland's mulslice front end on the host: the stacking-sequence parser
against the reference's own parlay() (oracle/_ref) and its documented examples."""
import ctypes
import os

import numpy as np
import pytest

from multislice_gb300.kirkland import StackingError, parlay

REF_LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                       "libkirkland_ref.so")
CASES = ["2(abc)d", "5( 2(abc) 3(cba) )", "abab", "10(ab)", "\t3(a\tb)c", "2(3(a)b)", "abe", "2ab", "(ab)",
         "ab)", "2(ab", "a-b", "ab  ", "12 (ab)", "0(ab)c", "ZzAa"]


def test_documented_examples():
    assert parlay("2(abc)d", 4) == [0, 1, 2, 0, 1, 2, 3]
    assert len(parlay("5( 2(abc) 3(cba) )", 3)) == 75
    with pytest.raises(StackingError) as e:
        parlay("2(ab", 2)
    assert e.value.code == -8


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="oracle/_ref not built (needs the reference tree)")
@pytest.mark.parametrize("seq", CASES)
def test_parlay_matches_reference(seq):
    lib = ctypes.CDLL(REF_LIB)
    out = np.zeros(4096, np.int32)
    n = ctypes.c_int(0)
    nlayer = 3
    rc = lib.kref_parlay(seq.encode(), out.ctypes.data, 4096, nlayer - 1, ctypes.byref(n))
    if rc == 0:
        assert parlay(seq, nlayer) == out[: n.value].tolist()
    else:
        with pytest.raises(StackingError) as e:
            parlay(seq, nlayer)
        assert e.value.code == rc
