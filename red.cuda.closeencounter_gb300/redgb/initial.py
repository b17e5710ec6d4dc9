"""The reference's initial-condition program as a command line: disks drawn on the GPU by
rg_populate_disks, written as the reference's body files.

    python -m redgb.initial {dvorak,n_gp,n_pp,n_spl,n_pl} [--n N] [--seed S] [--count C] -o PREFIX

writes PREFIX.txt (PREFIX_1.txt ... PREFIX_C.txt for C disks, seeds S .. S + C - 1), each a
body list in the format red.cuda reads (pp_disk.cu:1576-1612), like red.cuda.initial's
print(..., INPUT_FORMAT_RED).  The disks are the reference's set-ups (main.cu:88-385); N
replaces its body count.
"""
import argparse
import sys

from . import bodies
from .icgen import PRESETS, populate_disks, reference_preset


def main(argv=None):
    ap = argparse.ArgumentParser(prog="redgb.initial", description=__doc__.split("\n\n")[0])
    ap.add_argument("disk", choices=PRESETS)
    ap.add_argument("--n", type=int, default=None, help="bodies besides the star")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--count", type=int, default=1, help="disks to draw (seeds seed .. seed + count - 1)")
    ap.add_argument("-o", "--output", required=True, help="path prefix of the body files")
    a = ap.parse_args(argv)
    if a.count < 1 or (a.n is not None and a.n < 0):
        ap.error("--count must be positive and --n non-negative")
    specs = [reference_preset(a.disk, a.seed + k, a.n) for k in range(a.count)]
    try:
        disks = populate_disks(specs)
    except (RuntimeError, ValueError, OSError) as e:
        print(f"redgb.initial: {e}", file=sys.stderr)
        return 1
    paths = [f"{a.output}.txt"] if a.count == 1 else [f"{a.output}_{k + 1}.txt" for k in range(a.count)]
    for path, disk in zip(paths, disks):
        bodies.write_body_file(path, disk)
        print(path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
