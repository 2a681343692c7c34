"""Convert the reference's FPARAMS.DAT text table into fparams.npy.

FPARAMS.DAT (ImageSimulation/parserFPARAMS/FPARAMS.DAT:1-515) is Kirkland's
published 12-parameter fit of electron scattering factors: for every Z = 1..103
a header line "Z=  n,  chisq= x" followed by three lines of four numbers in
the order a1 b1 a2 b2 / a3 b3 c1 d1 / c2 d2 c3 d3 (the parser at
ImageSimulation/parserFPARAMS/main.cpp:18-98 reads the same order, and
LMultiSlice indexes it the same way at ModelPotential.cu:241-251).

The output is a float64 array of shape (104, 12); row Z holds the 12 numbers
for atomic number Z and row 0 is zero.  The product's C++ host parses the same
text format itself (msl_fparams_parse in include/msl.h); this script only
exists so the table travels with the package.

Usage: python make_fparams.py <path to FPARAMS.DAT> [out.npy]
"""
import os
import sys

import numpy as np


def parse_fparams_text(text):
    tab = np.zeros((104, 12), dtype=np.float64)
    lines = [ln.strip() for ln in text.splitlines()]
    i = 0
    seen = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("Z="):
            z = int(ln.split(",")[0].split("=")[1])
            vals = []
            j = i + 1
            while len(vals) < 12 and j < len(lines):
                if lines[j]:
                    vals.extend(float(v) for v in lines[j].split())
                j += 1
            if len(vals) != 12 or not (1 <= z <= 103):
                raise ValueError(f"bad FPARAMS record for Z={z}")
            tab[z] = vals
            seen += 1
            i = j
        else:
            i += 1
    if seen != 103:
        raise ValueError(f"expected 103 records, found {seen}")
    return tab


def main(argv):
    src = argv[1]
    out = argv[2] if len(argv) > 2 else os.path.join(os.path.dirname(__file__), "fparams.npy")
    with open(src, "r", encoding="latin-1") as f:
        tab = parse_fparams_text(f.read())
    np.save(out, tab)
    print(f"wrote {out}: {tab.shape}")


if __name__ == "__main__":
    main(sys.argv)
