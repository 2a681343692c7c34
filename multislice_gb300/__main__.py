"""Command line.

  python -m multislice_gb300 <job.xml> [--device N]
      Runs a reference job file (LMultiSlice <action> or the C# STEM driver's
      <Calculation_parameters>) on the GPU and writes its results next to it.
  python -m multislice_gb300 mulslice --layers a.tif b.tif --stack "40(ab)" --kev 200
      --out wave.tif [--start wave0.tif] [--cs A --df A --k-obj 1/A]
      Kirkland's mulslice: floatTIFF layer potentials and a stacking sequence in,
      the exit wave (or, with a lens, the CTEM image) out as floatTIFF.
"""
import argparse
import sys

from .jobs import run_job_file


def _mulslice(argv):
    from .api import Context
    from .kirkland import mulslice
    ap = argparse.ArgumentParser(prog="python -m multislice_gb300 mulslice")
    ap.add_argument("--layers", nargs="+", required=True)
    ap.add_argument("--stack", required=True)
    ap.add_argument("--kev", type=float, required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("--start")
    ap.add_argument("--cs", type=float)
    ap.add_argument("--df", type=float, default=0.0)
    ap.add_argument("--k-obj", type=float, default=1.0e3)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    lens = None if a.cs is None else dict(cs=a.cs, df=a.df, k_obj=a.k_obj)
    with Context(a.device) as ctx:
        _, seq = mulslice(ctx, a.layers, a.stack, a.kev, a.out, start_wave=a.start, lens=lens)
    print(f"{len(seq)} slices -> {a.out}")


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if argv and argv[0] == "mulslice":
        return _mulslice(argv[1:])
    ap = argparse.ArgumentParser(prog="python -m multislice_gb300")
    ap.add_argument("job", help="job XML file")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    res = run_job_file(args.job, args.device)
    for k, v in res.items():
        if isinstance(v, str):
            print(f"{k}: {v}")


if __name__ == "__main__":
    main()
