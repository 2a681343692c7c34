"""Convert the Doyle-Turner electron scattering-factor table of the reference's
Muslib into doyle_turner.npy and the C initialiser csrc/msl_doyle_turner.inc.

The table (Musli console 1.3 (STEM) 2/Muslib/Curves.cpp:86-179, the
`DoyleTurner bank[]` array) is the published four-Gaussian fit of Doyle &
Turner (Acta Cryst. A24, 390, 1968): for Z = 1..92 the pairs (a_j, b_j),
j = 1..4, of f(s) = sum_j a_j exp(-b_j s^2); row 0 is zero.  Each record in the
source reads `Z,"Sym",a1,b1,a2,b2,a3,b3,a4,b4,`.

Output: a float64 array of shape (93, 8), row Z = a1 b1 a2 b2 a3 b3 a4 b4, and
the same numbers as a C array for the library.

Usage: python make_doyle_turner.py <path to Curves.cpp>
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REC = re.compile(r'^\s*(\d+)\s*,\s*"([A-Za-z0-9]*)"\s*,((?:\s*-?[0-9.]+\s*,?){8})')


def parse(text):
    tab = np.zeros((93, 8), np.float64)
    seen = set()
    for ln in text.splitlines():
        m = REC.match(ln)
        if not m:
            continue
        z = int(m.group(1))
        vals = [float(v) for v in m.group(3).replace(" ", "").strip(",").split(",")]
        if len(vals) != 8 or z > 92:
            raise ValueError(f"bad Doyle-Turner record: {ln!r}")
        tab[z] = vals
        seen.add(z)
    if seen != set(range(93)):
        raise ValueError(f"expected records for Z = 0..92, found {len(seen)}")
    return tab


def main(argv):
    with open(argv[1], "r", encoding="latin-1") as f:
        tab = parse(f.read())
    np.save(os.path.join(HERE, "doyle_turner.npy"), tab)
    inc = os.path.join(HERE, "..", "csrc", "msl_doyle_turner.inc")
    with open(inc, "w") as f:
        f.write("// Generated by multislice_gb300/data/make_doyle_turner.py: Doyle & Turner (1968)\n"
                "// four-Gaussian electron scattering factors, row Z = a1 b1 a2 b2 a3 b3 a4 b4.\n")
        for z in range(93):
            f.write("    {" + ", ".join(repr(float(v)) for v in tab[z]) + "},\n")
    print(f"wrote doyle_turner.npy and msl_doyle_turner.inc: {tab.shape}")


if __name__ == "__main__":
    main(sys.argv)
