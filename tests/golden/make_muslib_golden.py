"""Generate tests/golden/muslib.npz from the reference's own Muslib code.

Muslib ("Musli console 1.3 (STEM) 2/Muslib": Curves.cpp, PG_RS.cpp, Pot_RS.cpp,
Pot_rec_DT_DW.cpp, Pot_rec_curve_DW.cpp, Propagator.cpp) is compiled unchanged
into oracle/_ref/libmuslib_ref.so by oracle/ref/Makefile, with a small
windows.h stand-in that keeps Windows' 32-bit long.  This script runs every
export the library replaces on small seeded inputs and stores inputs and
outputs, so the GPU exports (tests/test_gpu_muslib.py) and the numpy
restatement (tests/test_oracle_muslib.py) are checked against the reference's
own results:

  prop_*      CreatePropagator (Propagator.cpp:5-53) at two cell angles;
  rs_*        the sixteen PG_rs_* / Potential_rs_* forms (PG_RS.cpp, Pot_RS.cpp)
              at two cell angles, atoms whose boxes cross the cell edges;
  oneatom     PG_rs_curve_DW_cutpot_oneatom (PG_RS.cpp:5-55);
  rec_*       Potential_rec_DT_DW / Potential_rec_curve_DW (Pot_rec_*.cpp) for
              three (angle, multiplier, row band) cases;
  scat_*      scat_ampl_rs_DT_DW, scat_ampl_rs2_DT_DW(0), CreatePots_* (Curves.cpp).

Usage: python tests/golden/make_muslib_golden.py [reference root]
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

RS_FORMS = [(k, s, c, w) for k in ("PG", "Potential") for s in ("curve", "DT") for c in ("DW", "TV")
            for w in ("cutpot", "periodic")]
GAMS = (np.pi / 2, 1.8)


def p(a):
    return ctypes.c_void_p(a.ctypes.data)


def rs_inputs(src, coord, seed=9):
    """Seeded atoms on a 48 x 40 grid (the same generator the tests use)."""
    rng = np.random.default_rng(seed)
    a, b, E, atrad, N, M, na = 9.0, 10.5, 200e3, 1.8, 48, 40, 30
    xx, yy = rng.random(na), rng.random(na)
    xx[:4] = [0.01, 0.985, 0.5, 0.03]
    yy[:4] = [0.02, 0.97, 0.995, 0.5]
    if coord == "TV":
        xx, yy = xx * a, yy * b
    ads = rng.random(na) * 0.05
    occ = 0.5 + 0.5 * rng.random(na)
    dw = 0.2 + 0.6 * rng.random(na)
    if src == "curve":
        typ = rng.integers(0, 3, na).astype(np.int32)
        r = np.arange(300) * 0.01
        curves = np.ascontiguousarray(np.stack([z * np.exp(-r / 0.35) for z in (1.0, 2.0, 3.5)]))
    else:
        typ = rng.choice(np.array([8, 22, 38], np.int32), na)
        curves = np.zeros((0, 0))
    return dict(a=a, b=b, E=E, atrad=atrad, N=N, M=M, xx=xx, yy=yy, ads=ads, occ=occ, dw=dw, typ=typ,
                curves=curves)


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "-j8"], check=True,
                   capture_output=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmuslib_ref.so"))
    d = ctypes.c_double
    U = ctypes.c_uint32
    out = {}

    # propagator
    lib.CreatePropagator.argtypes = [d] * 7 + [U, U, ctypes.c_void_p, ctypes.c_void_p]
    for gi, gam in enumerate((np.pi / 2, 1.9)):
        a, b, dz, E, tx, ty, N, M = 12.0, 15.0, 2.5, 200e3, 0.003, -0.002, 48, 40
        gli = np.zeros((M, N, 2))
        cpro = ctypes.c_float(-1)
        assert lib.CreatePropagator(a, b, gam, dz, E, tx, ty, N, M, p(gli), ctypes.byref(cpro)) == 0
        out[f"prop_{gi}_args"] = np.array([a, b, gam, dz, E, tx, ty, N, M], np.float64)
        out[f"prop_{gi}_gli"] = gli
        out[f"prop_{gi}_cpro"] = np.float32(cpro.value)

    # real-space forms
    for kind, src, coord, wrap in RS_FORMS:
        name = f"{kind}_rs_{src}_{coord}_{wrap}"
        fn = getattr(lib, name)
        I = rs_inputs(src, coord)
        for gi, gam in enumerate(GAMS):
            N, M, na = I["N"], I["M"], len(I["xx"])
            gli = np.zeros((M, N, 2))
            if kind == "PG":
                gli[..., 0] = 1.0
            cpro = ctypes.c_float(0)
            head = [d(I["a"]), d(I["b"]), d(gam)] + ([d(I["E"])] if kind == "PG" else []) + [d(I["atrad"])]
            common = [U(N), U(M), U(na), p(I["xx"]), p(I["yy"])]
            if src == "curve":
                tail = [p(I["ads"]), p(I["occ"]), p(I["typ"]), p(I["curves"]), U(I["curves"].shape[1]),
                        d(0.01), p(gli), ctypes.byref(cpro)]
            elif coord == "DW":
                tail = [p(I["dw"]), p(I["ads"]), p(I["occ"]), p(I["typ"]), p(gli), ctypes.byref(cpro)]
            else:
                tail = [p(I["ads"]), p(I["occ"]), p(I["typ"]), p(gli), ctypes.byref(cpro)]
            assert fn(*head, *common, *tail) == 0, name
            out[f"rs_{name}_{gi}_gli"] = gli
            out[f"rs_{name}_{gi}_cpro"] = np.float32(cpro.value)
        for k in ("xx", "yy", "ads", "occ", "dw", "typ", "curves"):
            out[f"rsin_{src}_{coord}_{k}"] = I[k]
        out[f"rsin_{src}_{coord}_scalars"] = np.array([I["a"], I["b"], I["E"], I["atrad"], I["N"], I["M"]])

    # one atom
    a, b, gam, K, N, M = 8.0, 8.0, 1.9, 0.025, 48, 40
    r = np.arange(500) * 0.01
    cur = np.ascontiguousarray(4.0 * np.exp(-r / 0.5))
    gli = np.zeros((M, N, 2))
    gli[..., 0] = 1.0
    lib.PG_rs_curve_DW_cutpot_oneatom.argtypes = [d] * 5 + [U, U] + [d] * 4 + [ctypes.c_void_p, U, d,
                                                                               ctypes.c_void_p]
    assert lib.PG_rs_curve_DW_cutpot_oneatom(a, b, gam, K, 1.0, N, M, 0.3, 0.7, 0.04, 0.9, p(cur), 500,
                                             0.01, p(gli)) == 0
    out["oneatom_gli"] = gli
    out["oneatom_curve"] = cur

    # reciprocal space
    rng = np.random.default_rng(21)
    a, b, N, M, na = 11.0, 12.0, 48, 64, 40
    xx, yy = rng.random(na), rng.random(na)
    ads, occ = rng.random(na) * 0.05, 0.5 + 0.5 * rng.random(na)
    zs = np.array([8, 22, 38], np.int32)
    pick = rng.integers(0, 3, na)
    dwv = np.array([0.3, 0.45, 0.6])
    for k, v in dict(xx=xx, yy=yy, ads=ads, occ=occ, zs=zs, pick=pick, dwv=dwv).items():
        out[f"recin_{k}"] = v
    cases = [(np.pi / 2, (1, 1), (0, 64)), (1.75, (2, 1), (0, 40)), (np.pi / 2, (1, 3), (10, 60))]
    for ci, (gam, (Nm, Mm), (SL, EL)) in enumerate(cases):
        out[f"rec_{ci}_case"] = np.array([gam, Nm, Mm, SL, EL])
        for form in ("DT", "curve"):
            gli = np.zeros((EL - SL, N, 2))
            cpro = ctypes.c_float(0)
            if form == "DT":
                typ, DW = zs[pick], dwv[pick]
                rc = lib.Potential_rec_DT_DW(d(a), d(b), d(gam), U(Nm), U(Mm), U(N), U(M), U(na), U(SL), U(EL),
                                             p(xx), p(yy), p(DW), p(ads), p(occ), p(typ), p(gli),
                                             ctypes.byref(cpro))
            else:
                typ = pick.astype(np.int32)
                sc = np.zeros((3, 60))
                zz = zs.astype(np.int32)
                lib.CreatePots_rec_DT_DW(U(3), U(60), d(0.02), p(zz), p(dwv), d(1 / (a * b * np.sin(gam))), p(sc))
                out[f"rec_{ci}_curves"] = sc
                rc = lib.Potential_rec_curve_DW(d(a), d(b), d(gam), U(Nm), U(Mm), U(N), U(M), U(na), U(SL),
                                                U(EL), p(xx), p(yy), p(ads), p(occ), p(typ), p(sc), U(60),
                                                d(0.02), p(gli), ctypes.byref(cpro))
            assert rc == 0
            out[f"rec_{ci}_{form}_gli"] = gli
            out[f"rec_{ci}_{form}_cpro"] = np.float32(cpro.value)

    # scattering factors and curves
    for fn in ("scat_ampl_rs_DT_DW", "scat_ampl_rs2_DT_DW"):
        getattr(lib, fn).restype = d
        getattr(lib, fn).argtypes = [ctypes.c_int, d, d]
    lib.scat_ampl_rs2_DT_DW0.restype = d
    lib.scat_ampl_rs2_DT_DW0.argtypes = [ctypes.c_int, d]
    zq = np.array([1, 6, 8, 14, 22, 29, 38, 79, 92], np.int32)
    sq = np.array([0.0, 0.05, 0.3, 0.9, 2.0])
    tab = np.zeros((3, len(zq), len(sq)))
    for i, z in enumerate(zq):
        for j, s_ in enumerate(sq):
            tab[0, i, j] = lib.scat_ampl_rs_DT_DW(int(z), float(s_), 0.4)
            tab[1, i, j] = lib.scat_ampl_rs2_DT_DW(int(z), float(s_), 0.4)
            tab[2, i, j] = lib.scat_ampl_rs2_DT_DW0(int(z), float(s_))
    out["scat_z"], out["scat_s"], out["scat_tab"] = zq, sq, tab
    types = np.array([6, 29, 79], np.int32)
    dws = np.array([0.3, 0.5, 0.7])
    sc_rec, sc_rs = np.zeros((3, 80)), np.zeros((3, 80))
    lib.CreatePots_rec_DT_DW(U(3), U(80), d(0.015), p(types), p(dws), d(0.0123), p(sc_rec))
    lib.CreatePots_rs_DT_DW(U(3), U(80), d(0.015), p(types), p(dws), p(sc_rs))
    out["pots_types"], out["pots_dw"], out["pots_rec"], out["pots_rs"] = types, dws, sc_rec, sc_rs

    np.savez_compressed(os.path.join(HERE, "muslib.npz"), **out)
    print("wrote muslib.npz:", len(out), "arrays")


if __name__ == "__main__":
    main()
