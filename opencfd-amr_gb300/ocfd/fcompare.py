"""Compare two plotfiles zone by zone (the checks and output of
Util/Plotfile/fcompare.cpp):

    python -m ocfd.fcompare [-n|--norm 0|1|2] [-a|--allow_diff_grids]
                            [-r|--rel_tol rtol] [--abs_tol atol] file1 file2

Prints, per level, every variable's absolute error ||B - A|| and relative
error ||B - A|| / ||A||; exits 1 when a variable has a NaN or passes neither
tolerance (defaults 0: the files must be identical), else 0.
"""
from __future__ import annotations

import argparse
import sys


def main(argv=None):
    ap = argparse.ArgumentParser(prog="fcompare", add_help=True)
    ap.add_argument("-n", "--norm", type=int, default=0, choices=[0, 1, 2])
    ap.add_argument("-a", "--allow_diff_grids", action="store_true")
    ap.add_argument("-r", "--rel_tol", type=float, default=0.0)
    ap.add_argument("--abs_tol", type=float, default=0.0)
    ap.add_argument("file1")
    ap.add_argument("file2")
    a = ap.parse_args(argv)
    from .plotfile import compare
    r = compare(a.file1, a.file2, a.norm, a.allow_diff_grids)
    print("\n %24s  %24s  %24s" % ("variable name", "absolute error", "relative error"))
    print(" %24s  %24s  %24s" % ("", "(||A - B||)", "(||A - B||/||A||)"))
    print(" " + "-" * 76)
    ok = True
    for l in range(r["abs"].shape[0]):
        print(" level = %d" % l)
        for n, name in enumerate(r["names"]):
            nan = r["nan"][l, n]
            if nan:
                where = {1: "A", 2: "B", 3: "both A and B"}[int(nan)]
                print(" %-24s  < NaN present in %s >" % (name, where))
                ok = False
                continue
            ab, rel = r["abs"][l, n], r["rel"][l, n]
            print(" %-24s  %24.10g  %24.10g" % (name, ab, rel))
            ok = ok and (ab <= a.abs_tol or rel <= a.rel_tol)
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
