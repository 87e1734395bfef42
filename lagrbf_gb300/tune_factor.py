"""Measures the CTA size of the patch set-up / solve launch for each patch-size class on the
current GPU and writes the table lagrbf_gb300/csrc/lgb_factor_tune.h (then rebuild).

For each class (patches of up to 32, 64, ..., 2048 points and beyond) a synthetic 3D dataset whose
interior patches have about 3/4 of the class bound (jittered lattice, Wendland C2, ABC flow) is set
up with every CTA size (32, 64, 128, 256 threads, option factor_threads) from a fresh context, and
the event-timed set-up of all its patches (assembly, Cholesky, solves, record blocks) is compared;
the fastest size goes into the table.

    python -m lagrbf_gb300.tune_factor [--out PATH] [--repeat R]
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "csrc", "lgb_factor_tune.h")
THREADS = (32, 64, 128, 256)
NCLS = 8


def case(cls):
    """(data points, PU nodes per axis) with interior patches of about 3/4 of the class bound."""
    target = 0.75 * (32 << cls) if cls < NCLS - 1 else 3000.0
    ppc = target / 8.0                        # points per cell: a patch is 2 x 2 x 2 cells
    npu = 16 if cls <= 3 else (10 if cls <= 5 else 6)
    nlat = max(2, int(round((npu - 1) * ppc ** (1.0 / 3.0))))
    return nlat, npu


def time_setup(nlat, npu, threads, repeat):
    import lagrbf_gb300 as L
    from lagrbf_gb300 import workloads as W
    rng = np.random.default_rng(1)
    xd = W.jittered_lattice(nlat, 3, rng)
    fd = W.abc_flow(xd)
    xp = W.uniform_points(4 * (npu - 1) ** 3, 3, np.random.default_rng(2))
    best = None
    for _ in range(repeat):
        c = L.LagRBFCtx(dim=3, npartitions=[npu] * 3, overlap=W.pu_overlap(npu), shape_factor=1.0, kernel=2,
                        nfields=3, solve_method=2, eval_precision="fp32",
                        petsc_options={"factor_threads": threads, "setup_all_patches": True})
        c.fill_data(xd, fd)
        c.fill_points(xp)
        c.set_profiling(True)
        c.interpolate_c()
        st = c.stats()
        ms = st["factor_ms"]
        best = ms if best is None else min(best, ms)
        mp = st["max_patch"]
        del c
    return best, mp


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--repeat", type=int, default=2)
    args = ap.parse_args()
    table, rows = [], []
    for cls in range(NCLS):
        nlat, npu = case(cls)
        times = {}
        for t in THREADS:
            times[t], mp = time_setup(nlat, npu, t, args.repeat)
        best = min(times, key=times.get)
        table.append(best)
        rows.append({"class": cls, "bound": (32 << cls) if cls < NCLS - 1 else None, "nlat": nlat, "npu": npu,
                     "max_patch": mp, "setup_ms": times, "best": best})
        print(json.dumps(rows[-1]), flush=True)
    lines = ["/*",
             " * lgb_factor_tune.h -- CTA size of the patch set-up / solve launch of each patch-size class",
             " * (classes of up to 32, 64, 128, 256, 512, 1024, 2048 points and beyond), measured by",
             " *     python -m lagrbf_gb300.tune_factor",
             " * (event-timed set-up of every patch of a synthetic dataset per class, CTA sizes 32-256):"]
    for r in rows:
        lines.append(" *   class %d (%s): %s -> %d" % (r["class"], "<= %d" % r["bound"] if r["bound"] else "larger",
                                                       ", ".join("%d: %.1f ms" % (k, v) for k, v in r["setup_ms"].items()),
                                                       r["best"]))
    lines += [" */", "#ifndef LGB_FACTOR_TUNE_H", "#define LGB_FACTOR_TUNE_H",
              "static const int lgb_factor_threads[LGB_NCLS] = {%s};" % ", ".join(str(t) for t in table), "#endif", ""]
    with open(args.out, "w") as f:
        f.write("\n".join(lines))
    print("wrote", args.out)
    return 0


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    sys.exit(main())
