"""Command line: python -m multislice_gb300 <job.xml> [--device N]

Runs a reference job file (LMultiSlice <action> or the C# STEM driver's
<Calculation_parameters>) on the GPU and writes MRC results next to it."""
import argparse

from .jobs import run_job_file


def main(argv=None):
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
