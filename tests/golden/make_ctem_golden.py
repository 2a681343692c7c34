"""Generate tests/golden/ctem_partial.npz from the reference's own CTEM imaging code.

Runs the partial-coherence image of Kirkland's mulslice (mulslice.cpp:539-676,
restated as kref_partial_coherence in oracle/ref/kirkland_ref.cpp around the
reference's cfpix transforms and propagate(), compiled unchanged by
oracle/ref/Makefile) on the Si 64^2 case of tests/golden/si_small.npz, and the
reference's aberration function chi() (slicelib.cpp:258-323) on a grid of
angles:

  pc_<case>_pix    image [64][64] (float32) and its angle count for
                   case 0: illumination angles 0..6 mrad, defocus spread 30 A
                           (step 15 A), 2- and 3-fold astigmatism;
                   case 1: one angle (acmax = 0), defocus spread 40 A (step 20 A);
                   case 2: one angle, one defocus (the coherent image);
  chi_*            chi() for Cs, defocus, C12a/b and C23a/b at angles (alx, aly).

Usage: python tests/golden/make_ctem_golden.py [reference root]
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

# (acmin, acmax) mrad, Cs mm, df0, sigmaf, dfdelt A, aobj mrad, dfa2 A, dfa2phi deg, dfa3 A, dfa3phi deg
CASES = [
    (0.0, 6.0, 1.2, -600.0, 30.0, 15.0, 20.0, 40.0, 20.0, 300.0, 40.0),
    (0.0, 0.0, 1.2, -600.0, 40.0, 20.0, 25.0, 0.0, 0.0, 0.0, 0.0),
    (0.0, 0.0, 0.5, 300.0, 0.0, 1.0, 30.0, 25.0, 60.0, 150.0, 10.0),
]


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "-j8"], check=True,
                   capture_output=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libkirkland_ref.so"))
    d, vp = ctypes.c_double, ctypes.c_void_p
    lib.kref_partial_coherence.argtypes = ([ctypes.c_int, ctypes.c_int, d, d, d, ctypes.c_int, vp, vp,
                                            ctypes.c_int, vp] + [d] * 11 + [vp, vp])
    lib.kref_chi.restype = d
    lib.kref_chi.argtypes = [vp, d, d, ctypes.c_int]
    G = np.load(os.path.join(HERE, "si_small.npz"))
    vz = np.ascontiguousarray(G["v"], np.float64)
    nl, nx, ny = vz.shape
    cz = np.full(nl, float(G["dz"]))
    seq = np.ascontiguousarray(G["seq"], np.int32)
    out = {"cases": np.array(CASES)}
    for ci, c in enumerate(CASES):
        acmin, acmax, cs, df0, sigf, dfd, aobj, dfa2, dfa2p, dfa3, dfa3p = c
        pix = np.zeros((nx, ny), np.float32)
        nill = ctypes.c_int(0)
        assert lib.kref_partial_coherence(nx, ny, float(G["ax"]), float(G["by"]), float(G["kev"]), nl,
                                          vz.ctypes.data, cz.ctypes.data, len(seq), seq.ctypes.data, cs, df0,
                                          sigf, dfd, aobj, acmin, acmax, dfa2, dfa2p, dfa3, dfa3p,
                                          pix.ctypes.data, ctypes.byref(nill)) == 0
        out[f"pc_{ci}_pix"] = pix
        out[f"pc_{ci}_nillum"] = np.int32(nill.value)

    # chi(): Cs, defocus, two-fold and three-fold astigmatism coefficients
    npar = lib.kref_nparam()
    idx = [lib.kref_param_index(i) for i in range(6)]
    coef = np.array([1.2e7, -600.0, 30.0, -25.0, 400.0, 250.0])
    p = np.zeros(npar, np.float32)
    for i, v in zip(idx, coef):
        p[i] = v
    al = np.linspace(-0.02, 0.02, 9)
    alx, aly = np.meshgrid(al, al * 0.7 + 0.003, indexing="ij")
    w = np.array([[lib.kref_chi(p.ctypes.data, float(x), float(y), 1) for x, y in zip(rx, ry)]
                  for rx, ry in zip(alx, aly)])
    out["chi_coef"], out["chi_alx"], out["chi_aly"], out["chi_w"] = coef, alx, aly, w
    np.savez_compressed(os.path.join(HERE, "ctem_partial.npz"), **out)
    print("wrote ctem_partial.npz:", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
